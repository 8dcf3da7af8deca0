// grid.cu - cell-list neighbour search (Computer::SearchNeighbor, Computer.hpp:698-756;
// Grid::Store / Grid::Iterator, Grid.hpp:276-559).
//
// The reference stores particles serially (ascending index) into dense cells and
// then walks the nine surrounding cells in a fixed order.  Here every particle
// claims a slot of its cell with one atomic, each cell is then sorted back to
// ascending index (so the slot order equals the serial insertion order), and one
// thread per particle walks the nine cells and writes its list into the
// transposed ELL array.  The output equals the reference's list element for
// element: same candidates, same order, same distance test.
//
// Compiled with -fmad=false: the distance test must round exactly like the
// reference's sqrt(inner_prod(r, r)) < NeighborLength.
#include "common.cuh"

namespace mpsgb {

// Grid::Block (Grid.hpp:250-254) + Grid::Store (:276-331): out-of-domain particles
// are disabled (Computer.hpp:710-715); a cell beyond maxPerCell is the reference's
// "Too many particle in a block" error.
__global__ void k_bucket(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    st.x32[i] = __double2float_rn(st.x[i]);
    st.z32[i] = __double2float_rn(st.z[i]);
    st.cell_xz[i] = -1;
    if (st.unplaced) st.unplaced[i] = 1;
    if (st.type[i] == MPS_TYPE_DISABLED) {
        atomicAdd(&st.status->disabled, 1);
        return;
    }
    const double fx = floor(__ddiv_rn(__dadd_rn(st.x[i], -sc.min_x), sc.nl));
    const double fz = floor(__ddiv_rn(__dadd_rn(st.z[i], -sc.min_z), sc.nl));
    if (!(fx >= 0.0 && fx < static_cast<double>(sc.gnx) && fz >= 0.0 &&
          fz < static_cast<double>(sc.gnz))) {
        st.type[i] = MPS_TYPE_DISABLED;
        atomicAdd(&st.status->disabled, 1);
        return;
    }
    const int base = st.scene_of ? st.scene_of[i] * sc.cells_per_scene : 0;
    const int cell = base + static_cast<int>(fx) * sc.gnz + static_cast<int>(fz);
    const int slot = atomicAdd(&st.cell_count[cell], 1);
    if (slot < sc.max_per_cell) {
        st.cell_slot[static_cast<int64_t>(cell) * sc.max_per_cell + slot] = i;
        st.cell_xz[i] = (static_cast<int>(fx) << 16) | static_cast<int>(fz);
        if (st.unplaced) st.unplaced[i] = 0;
    } else {
        atomicOr(&st.status->flags, kStatusCellOverflow);
    }
}

// Restores the serial insertion order of each cell (ascending particle index).
__global__ void k_cell_sort(SceneConst sc, DeviceState st) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= sc.cells_per_scene * sc.nscenes) return;
    const int cnt = min(st.cell_count[c], sc.max_per_cell);
    if (st.cell_fill) st.cell_fill[c] = cnt;
    if (cnt < 2) return;
    int32_t* s = st.cell_slot + static_cast<int64_t>(c) * sc.max_per_cell;
    int buf[64];
    const int m = min(cnt, 64);
    for (int a = 0; a < m; a++) buf[a] = s[a];
    for (int a = 1; a < m; a++) {
        const int v = buf[a];
        int b = a - 1;
        while (b >= 0 && buf[b] > v) {
            buf[b + 1] = buf[b];
            b--;
        }
        buf[b + 1] = v;
    }
    if (cnt > 64) {  // maxPerCell > 64 only for r_e/l0 beyond 6: fall back to in-place sort
        for (int a = 1; a < cnt; a++) {
            const int v = s[a];
            int b = a - 1;
            while (b >= 0 && s[b] > v) {
                s[b + 1] = s[b];
                b--;
            }
            s[b + 1] = v;
        }
        return;
    }
    for (int a = 0; a < m; a++) s[a] = buf[a];
}

// Neighbour rows: the nine cells in Grid::Iterator order (Grid.hpp:393-401), each in
// slot order, keeping j != i with R(x_i, x_j) < NeighborLength (Computer.hpp:740-749).
// The FP32 range class settles almost every candidate; the rest take the FP64 test.
__device__ __forceinline__ int neighbor_row(const SceneConst& sc, const DeviceState& st, int i) {
    const double xi = st.x[i], zi = st.z[i];
    const float xi32 = st.x32[i], zi32 = st.z32[i];
    const float si32 = fabsf(xi32) + fabsf(zi32);
    const int bx = static_cast<int>(floor(__ddiv_rn(__dadd_rn(xi, -sc.min_x), sc.nl)));
    const int bz = static_cast<int>(floor(__ddiv_rn(__dadd_rn(zi, -sc.min_z), sc.nl)));
    const int base = st.scene_of ? st.scene_of[i] * sc.cells_per_scene : 0;
    int cnt = 0;
    for (int di = -1; di <= 1; di++) {
        const int cx = bx + di;
        if (cx < 0 || cx >= sc.gnx) continue;
        for (int dk = -1; dk <= 1; dk++) {
            const int cz = bz + dk;
            if (cz < 0 || cz >= sc.gnz) continue;
            const int cell = base + cx * sc.gnz + cz;
            const int m = min(st.cell_count[cell], sc.max_per_cell);
            const int32_t* slots = st.cell_slot + static_cast<int64_t>(cell) * sc.max_per_cell;
            for (int l = 0; l < m; l++) {
                const int j = slots[l];
                if (j == i) continue;
                const int cls = range_class(xi32, zi32, si32, st.x32[j], st.z32[j], sc.f32_in_nl,
                                            sc.f32_out_nl);
                bool inside = cls == 1;
                if (cls == 2) {
                    const double dx = __dadd_rn(xi, -st.x[j]);
                    const double dz = __dadd_rn(zi, -st.z[j]);
                    const double r2 = dot2(dx, dz, dx, dz);
                    if (r2 < sc.nl2_lo) {
                        inside = true;
                    } else if (r2 > sc.nl2_hi) {
                        inside = false;
                    } else {
                        inside = __dsqrt_rn(r2) < sc.nl;
                    }
                }
                if (inside) {
                    if (cnt < sc.nb_stride) {
                        st.nb[ell(cnt, sc.n, i)] = j;
                    } else {
                        atomicOr(&st.status->flags, kStatusDeviceCheck);
                        st.status->check_index = i;
                    }
                    cnt++;
                }
            }
        }
    }
    return min(cnt, sc.nb_stride);
}

__global__ void k_neighbors(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int cnt = 0;
    if (i < sc.n && st.type[i] != MPS_TYPE_DISABLED) cnt = neighbor_row(sc, st, i);
    if (i < sc.n) st.nb_count[i] = cnt;
    warp_add_u64(&st.status->nb_total, static_cast<unsigned long long>(cnt));
}

// Rows of the PPE: cell c's particles take rows cell_start[c] .. in slot order, particles
// without a slot follow all of them in index order.  Threads [0, cells) walk the cells,
// the rest the particles.
__global__ void k_rows(SceneConst sc, DeviceState st, int cells) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cells) {
        const int fill = st.cell_fill[t];
        const int r0 = st.cell_start[t];
        const int code = ((t / sc.gnz) << 16) | (t - (t / sc.gnz) * sc.gnz);
        const int32_t* slots = st.cell_slot + static_cast<int64_t>(t) * sc.max_per_cell;
        for (int k = 0; k < fill; k++) {
            const int i = slots[k];
            st.row_of[i] = r0 + k;
            st.particle_of[r0 + k] = i;
            st.row_cell[r0 + k] = code;
        }
        return;
    }
    const int i = t - cells;
    if (i >= sc.n || !st.unplaced[i]) return;
    const int r = st.cell_start[cells] + st.unplaced_pos[i];
    st.row_of[i] = r;
    st.particle_of[r] = i;
    st.row_cell[r] = -1;
}

// Zeroes the per-step counters of the status block and keeps its failure flags.
__global__ void k_status_counters_reset(DevStatus* st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->disabled = 0;
        st->nb_total = 0;
        st->ppe_nnz = 0;
    }
}

void launch_status_counters_reset(DevStatus* st, cudaStream_t s) { k_status_counters_reset<<<1, 32, 0, s>>>(st); }

// FP32 copies of the positions of particles [first, first + count) after a host write of
// x, z (and y in 3D).
__global__ void k_positions_f32(DeviceState st, int first, int count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = first + k;
    st.x32[i] = __double2float_rn(st.x[i]);
    st.z32[i] = __double2float_rn(st.z[i]);
    if (st.y32) st.y32[i] = __double2float_rn(st.y[i]);
}

void launch_positions_f32(const SceneConst& sc, const DeviceState& st, cudaStream_t s, int first, int count) {
    if (count < 0) count = sc.n - first;
    if (count <= 0) return;
    k_positions_f32<<<grid_for(count), kBlock, 0, s>>>(st, first, count);
}

void launch_bucket(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_bucket<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_cell_sort(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_cell_sort<<<grid_for(static_cast<int64_t>(sc.cells_per_scene) * sc.nscenes), kBlock, 0, s>>>(sc, st);
}

void launch_neighbors(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_neighbors<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
}

int launch_rows(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    if (!st.row_of) return 0;
    const int cells = sc.cells_per_scene;
    launch_exclusive_scan(st.cell_fill, st.cell_start, cells, st.row_scratch, s);
    launch_exclusive_scan(st.unplaced, st.unplaced_pos, sc.n, st.row_scratch, s);
    k_rows<<<grid_for(static_cast<int64_t>(cells) + sc.n), kBlock, 0, s>>>(sc, st, cells);
    return 7;
}

}  // namespace mpsgb
