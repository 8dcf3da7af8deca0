// dim3.cu - the time step of a three-dimensional scene (DIM3, defines.hpp:9-11 and the
// DIM3 branches of Grid.hpp, Environment.hpp and Computer.hpp): neighbour search over
// the 27 surrounding cells, number density, error-compensating source, explicit forces,
// SaveX, PPE assembly, pressure gradient (plain and GC), dynamic stabilisation and the
// CFL time step.
//
// The kernels follow the two-dimensional ones of grid.cu and stages.cu: one thread per
// particle walks its neighbour row in reference order and accumulates like
// AccumulateNeighbor (Computer.hpp:618-695), with the filter r^2 < r_e^2, the terms in
// list order and the SPP particle last.  Vectors have three components, summed in the
// reference's order (uBLAS inner_prod and prod run each sum from 0), and DIM = 3 enters
// the coefficients as in the reference: nu (5 - DIM) r_e / n0 / r^3, 2 DIM / lambda / n0,
// -dt / rho DIM / n0, DIM / n0 for the GC identity.  The range tests take the FP32
// screen of the 2D kernels on three coordinates (range_class3 / for_near3: surely-in and
// surely-out pairs settled in FP32, the rest by the reference's FP64 test, so every
// decision is the FP64 one).  Compiled with -fmad=false: results are bit-identical to the
// FP64 CPU path.  The PPE rows are the particles in index order; the layout kernels, the
// pressure assignment, the explicit pressure and the solvers are the dimension-free
// ones.
#include "common.cuh"

namespace mpsgb {

namespace {

// uBLAS inner_prod of 3-vectors: ((0 + a0 b0) + a1 b1) + a2 b2
__device__ __forceinline__ double dot3(double a0, double a1, double a2, double b0, double b1, double b2) {
    return __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(a0, b0)), __dmul_rn(a1, b1)), __dmul_rn(a2, b2));
}

// dot3 without its leading 0 + (see dot2_term in common.cuh)
__device__ __forceinline__ double dot3_term(double a0, double a1, double a2, double b0, double b1, double b2) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1)), __dmul_rn(a2, b2));
}

// inner_prod(d, d) without the 0 + (a square is never -0)
__device__ __forceinline__ double dist3(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ bool is_surface3(const SceneConst& sc, double nd) {
    return ddiv_rn(nd, sc.n0) < sc.surface_ratio;  // Computer.hpp:586-589
}

// FP32 copies of particle i's position (the range screen reads them).
__device__ __forceinline__ void positions_f32(const DeviceState& st, int i) {
    st.x32[i] = __double2float_rn(st.x[i]);
    st.y32[i] = __double2float_rn(st.y[i]);
    st.z32[i] = __double2float_rn(st.z[i]);
}

// ------------------------------------------------------------------ search
// Grid::Block + Grid::Store (Grid.hpp:250-331), cells [x][y][z]; out-of-domain particles
// are disabled (Computer.hpp:710-715).
__global__ void k3_bucket(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    st.x32[i] = __double2float_rn(st.x[i]);
    st.y32[i] = __double2float_rn(st.y[i]);
    st.z32[i] = __double2float_rn(st.z[i]);
    if (st.type[i] == MPS_TYPE_DISABLED) {
        atomicAdd(&st.status->disabled, 1);
        return;
    }
    const double fx = floor(ddiv_rn(__dadd_rn(st.x[i], -sc.min_x), sc.nl));
    const double fy = floor(ddiv_rn(__dadd_rn(st.y[i], -sc.min_y), sc.nl));
    const double fz = floor(ddiv_rn(__dadd_rn(st.z[i], -sc.min_z), sc.nl));
    if (!(fx >= 0.0 && fx < static_cast<double>(sc.gnx) && fy >= 0.0 && fy < static_cast<double>(sc.gny) &&
          fz >= 0.0 && fz < static_cast<double>(sc.gnz))) {
        st.type[i] = MPS_TYPE_DISABLED;
        atomicAdd(&st.status->disabled, 1);
        return;
    }
    const int cell = (static_cast<int>(fx) * sc.gny + static_cast<int>(fy)) * sc.gnz + static_cast<int>(fz);
    const int slot = atomicAdd(&st.cell_count[cell], 1);
    if (slot < sc.max_per_cell)
        st.cell_slot[static_cast<int64_t>(cell) * sc.max_per_cell + slot] = i;
    else
        atomicOr(&st.status->flags, kStatusCellOverflow);
}

// SearchNeighbor (Computer.hpp:720-755): the 27 cells in Grid::Iterator order (x, then y,
// then z from -1 to +1, Grid.hpp:364-391), each in slot (ascending index) order; j != i
// with R(x_i, x_j) < NeighborLength.  The row holds 9 maxPerCell entries, the
// reference's MaxNeighborCount (Computer.hpp:1136-1140); an entry beyond it is a device
// check error (the reference would write past its row).
__global__ void k3_neighbors(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int cnt = 0;
    if (i < sc.n && st.type[i] != MPS_TYPE_DISABLED) {
        const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
        const float xi32 = st.x32[i], yi32 = st.y32[i], zi32 = st.z32[i];
        const float si32 = (fabsf(xi32) + fabsf(yi32)) + fabsf(zi32);
        const int bx = static_cast<int>(floor(ddiv_rn(__dadd_rn(xi, -sc.min_x), sc.nl)));
        const int by = static_cast<int>(floor(ddiv_rn(__dadd_rn(yi, -sc.min_y), sc.nl)));
        const int bz = static_cast<int>(floor(ddiv_rn(__dadd_rn(zi, -sc.min_z), sc.nl)));
        for (int di = -1; di <= 1; di++) {
            const int cx = bx + di;
            if (cx < 0 || cx >= sc.gnx) continue;
            for (int dj = -1; dj <= 1; dj++) {
                const int cy = by + dj;
                if (cy < 0 || cy >= sc.gny) continue;
                for (int dk = -1; dk <= 1; dk++) {
                    const int cz = bz + dk;
                    if (cz < 0 || cz >= sc.gnz) continue;
                    const int cell = (cx * sc.gny + cy) * sc.gnz + cz;
                    const int m = min(st.cell_count[cell], sc.max_per_cell);
                    const int32_t* slots = st.cell_slot + static_cast<int64_t>(cell) * sc.max_per_cell;
                    for (int l = 0; l < m; l++) {
                        const int j = slots[l];
                        if (j == i) continue;
                        const int cls = range_class3(xi32, yi32, zi32, si32, st.x32[j], st.y32[j], st.z32[j],
                                                     sc.f32_in_nl, sc.f32_out_nl);
                        bool inside = cls == 1;
                        if (cls == 2) {  // the FP64 test, the square root only near NL
                            const double dx = __dadd_rn(xi, -st.x[j]);
                            const double dy = __dadd_rn(yi, -st.y[j]);
                            const double dz = __dadd_rn(zi, -st.z[j]);
                            const double r2 = dist3(dx, dy, dz);
                            inside = (r2 < sc.nl2_lo) ? true : (r2 > sc.nl2_hi) ? false : dsqrt_rn(r2) < sc.nl;
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
        }
        cnt = min(cnt, sc.nb_stride);
    }
    if (i < sc.n) st.nb_count[i] = cnt;
    warp_add_u64(&st.status->nb_total, static_cast<unsigned long long>(cnt));
}

// ------------------------------------------------------------------ helpers
// The SPP particle (Computer.hpp:664-692); (gx, gy, gz) holds sum W(r) dx over the
// neighbours within `radius`.
__device__ __forceinline__ bool spp_particle3(const SceneConst& sc, const DeviceState& st, int i, double radius,
                                              double gx, double gy, double gz, double& xs, double& ys,
                                              double& zs) {
    const double thisN = st.n_wo_spp[i];
    gx = ddiv_rn(gx, sc.n0);
    gy = ddiv_rn(gy, sc.n0);
    gz = ddiv_rn(gz, sc.n0);
    if (thisN < sc.n0) {
        const double r_g = dsqrt_rn(dot3(gx, gy, gz, gx, gy, gz));
        if (r_g > 2.220446049250313080847e-16) {  // std::numeric_limits<double>::epsilon()
            const double w_spp = __dadd_rn(sc.n0, -thisN);
            const double r_spp = ddiv_rn(radius, __dadd_rn(w_spp, 1.0));
            const double s = ddiv_rn(r_spp, r_g);
            xs = __dadd_rn(st.x[i], -__dmul_rn(s, gx));
            ys = __dadd_rn(st.y[i], -__dmul_rn(s, gy));
            zs = __dadd_rn(st.z[i], -__dmul_rn(s, gz));
            return true;
        }
    }
    return false;
}

// The Laplacian factors with DIM = 3, in the reference's left-to-right order:
// viscosity HL ((nu 2) re_lap) / n0_lap, else (((nu 2) 3) / lambda_lap) / n0_lap;
// PPE HL (2 re_lap) / n0_lap, else (6 / lambda_lap) / n0_lap.
struct LapFactors3 {
    bool hl;
    double visc, ppe;
};
__device__ __forceinline__ LapFactors3 lap_factors3(const SceneConst& sc) {
    LapFactors3 f;
    f.hl = has_flag(sc.flags, MPS_FLAG_HL);
    f.visc = f.hl ? sc.nu * 2.0 * sc.re_lap / sc.n0_lap : sc.nu * 2 * 3.0 / sc.lambda_lap / sc.n0_lap;
    f.ppe = f.hl ? 2.0 * sc.re_lap / sc.n0_lap : 6.0 / sc.lambda_lap / sc.n0_lap;
    return f;
}
__device__ __forceinline__ double viscosity_coefficient3(const SceneConst& sc, const LapFactors3& f, double r) {
    if (f.hl) return ddiv_rn(f.visc, r * r * r);  // Computer.hpp:963-970
    return f.visc * weight(r, sc.re_lap);
}
__device__ __forceinline__ double ppe_coefficient3(const SceneConst& sc, const LapFactors3& f, double r) {
    if (f.hl) return ddiv_rn(f.ppe, r * r * r);  // Computer.hpp:1290-1297
    return f.ppe * weight(r, sc.re_lap);
}

// NeighborDensityVariationSpeed (Computer.hpp:838-872)
__device__ double density_variation3(const SceneConst& sc, const DeviceState& st, int i, double dt) {
    if (has_flag(sc.flags, MPS_FLAG_HS)) {
        if (has_flag(sc.flags, MPS_FLAG_SPP) && st.n_wo_spp[i] < sc.n0) return 0.0;
        const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
        const double ui = st.u[i], vi = st.v[i], wi = st.w[i];
        double sum = 0.0;
            for_near3(sc, st, i, sc.f32_out_re, [&](int j) {
            const double dx = st.x[j] - xi;
            const double dy = st.y[j] - yi;
            const double dz = st.z[j] - zi;
            const double r2 = dist3(dx, dy, dz);
            if (below(r2, sc.re2)) {
                const double du = st.u[j] - ui;
                const double dv = st.v[j] - vi;
                const double dw = st.w[j] - wi;
                const double r = dsqrt_rn(r2);
                sum += ddiv_rn(dot3_term(dx, dy, dz, du, dv, dw), r * r * r);
            }
        });
        return -sc.re * sum;
    }
    return (st.nd[i] - sc.n0) / dt;
}

// ------------------------------------------------------------------ stages
// DetermineDt (Computer.hpp:759-777), part 1: max |u|^2 (part 2 is k_cfl_dt).
__global__ void k3_max_speed(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < sc.n) v = dot3(st.u[i], st.v[i], st.w[i], st.u[i], st.v[i], st.w[i]);
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0)
        atomicMax(&st.step->max_u2_bits, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// ComputeNeighborDensities (Computer.hpp:780-833)
__global__ void k3_density(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    if (spp) st.n_wo_spp[i] = sc.n0;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
    double thisN = 0.0;
    for_near3(sc, st, i, sc.f32_out_re, [&](int j) {
        const double r2 = dist3(st.x[j] - xi, st.y[j] - yi, st.z[j] - zi);
        if (below(r2, sc.re2)) thisN += weight(dsqrt_rn(r2), sc.re);
    });
    if (spp) {
        st.n_wo_spp[i] = thisN;
        st.nd[i] = (thisN < sc.n0) ? sc.n0 : thisN;
    } else {
        st.nd[i] = thisN;
    }
}

// ComputeErrorCorrection (Computer.hpp:877-910)
__global__ void k3_error_correction(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const double speed = density_variation3(sc, st, i, st.step->dt);
    const double error = (st.nd[i] - sc.n0) / sc.n0;
    st.ecs[i] = fabs(error) * speed + fabs(speed) * error;
}

__global__ void k3_density_variation(SceneConst sc, DeviceState st, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    const int t = st.type[i];
    out[i] = (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) ? 0.0 : density_variation3(sc, st, i, st.step->dt);
}

// ComputeExplicitForces, first loop (Computer.hpp:935-990): a = viscosity + G, G = (0, 0, -g).
__global__ void k3_explicit_accel(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const LapFactors3 lf = lap_factors3(sc);
    const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
    const double ui = st.u[i], vi = st.v[i], wi = st.w[i];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for_near3(sc, st, i, sc.f32_out_rl, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dy = st.y[j] - yi;
        const double dz = st.z[j] - zi;
        const double r2 = dist3(dx, dy, dz);
        if (!below(r2, sc.rl2)) return;
        if (st.type[j] != MPS_TYPE_DUMMY) {
            const double c = viscosity_coefficient3(sc, lf, dsqrt_rn(r2));
            ax += c * (st.u[j] - ui);
            ay += c * (st.v[j] - vi);
            az += c * (st.w[j] - wi);
        }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
    });
    // With SPP the reference adds the virtual particle's viscosity term c (u_i - u_i),
    // which is +0 for finite velocities: the virtual particle is not built here
    // (sums_from_zero, common.cuh).
    if (has_flag(sc.flags, MPS_FLAG_CENTRAL_GRAVITY)) {  // Computer.hpp:981-988
        const double g = -sc.g;
        const double r = dsqrt_rn(dot3(xi, yi, zi, xi, yi, zi));
        double cx = 0.0, cy = 0.0, cz = 0.0;
        if (!(r < sc.l0 * 0.01)) {
            cx = xi / r;
            cy = yi / r;
            cz = zi / r;
        }
        st.dux[i] = ax + g * cx;
        st.duy[i] = ay + g * cy;
        st.duz[i] = az + g * cz;
    } else {
        st.dux[i] = __dadd_rn(ax, 0.0);
        st.duy[i] = __dadd_rn(ay, 0.0);
        st.duz[i] = az + (-sc.g);
    }
}

// ComputeExplicitForces, second loop (Computer.hpp:995-1020).
__global__ void k3_explicit_update(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const double dt = st.step->dt;
    if (st.type[i] == MPS_TYPE_FLUID) {
        const double u = st.u[i] + st.dux[i] * dt;
        const double v = st.v[i] + st.duy[i] * dt;
        const double w = st.w[i] + st.duz[i] * dt;
        st.u[i] = u;
        st.v[i] = v;
        st.w[i] = w;
        st.x[i] = st.x[i] + u * dt;
        st.y[i] = st.y[i] + v * dt;
        st.z[i] = st.z[i] + w * dt;
    } else {
        const double nx = st.wall_x[i], ny = st.wall_y[i], nz = st.wall_z[i];
        st.u[i] = (nx - st.x[i]) / dt;
        st.v[i] = (ny - st.y[i]) / dt;
        st.w[i] = (nz - st.z[i]) / dt;
        st.x[i] = nx;
        st.y[i] = ny;
        st.z[i] = nz;
    }
    positions_f32(st, i);
}

// SaveX (Computer.hpp:1025-1039)
__global__ void k3_save_x(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    st.ox[i] = st.x[i];
    st.oy[i] = st.y[i];
    st.oz[i] = st.z[i];
}

// SetPressurePoissonEquation (Computer.hpp:1145-1328) into the scratch ELL arrays, rows
// in particle order (diagonal last).
__global__ void k3_ppe_build(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const int n = sc.n;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED || (!spp && is_surface3(sc, st.nd[i]))) {
        st.ppe_b[i] = 0;
        st.ppe_x[i] = 0;
        st.ppe_col_tmp[ell(0, n, i)] = i;
        st.ppe_val_tmp[ell(0, n, i)] = 1.0;
        st.ppe_len[i] = 1;
        return;
    }
    const LapFactors3 lf = lap_factors3(sc);
    const double dt = st.step->dt;
    const double speed = density_variation3(sc, st, i, dt);
    if (has_flag(sc.flags, MPS_FLAG_ECS)) {
        const double e = st.ecs[i];
        st.ppe_b[i] = -sc.rho / (sc.n0 * dt) * (speed + e);
    } else {
        st.ppe_b[i] = -sc.rho / (sc.n0 * dt) * speed;
    }
    st.ppe_x[i] = st.p[i];
    const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
    double a_ii = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    int m = 0;
    for_near3(sc, st, i, sc.f32_out_rl, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dy = st.y[j] - yi;
        const double dz = st.z[j] - zi;
        const double r2 = dist3(dx, dy, dz);
        if (!below(r2, sc.rl2)) return;
        if (st.type[j] != MPS_TYPE_DUMMY) {
            const double a_ij = ppe_coefficient3(sc, lf, dsqrt_rn(r2));
            if (spp || !is_surface3(sc, st.nd[j])) {
                st.ppe_col_tmp[ell(m, n, i)] = j;
                st.ppe_val_tmp[ell(m, n, i)] = a_ij;
                m++;
            }
            a_ii += -a_ij;
        }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        if (spp) {
            const double wg = weight(dsqrt_rn(r2), sc.re_lap);
            gx += wg * dx;
            gy += wg * dy;
            gz += wg * dz;
        }
    });
    double xs, ys, zs;
    if (spp && spp_particle3(sc, st, i, sc.re_lap, gx, gy, gz, xs, ys, zs)) {
        const double ddx = xi - xs, ddy = yi - ys, ddz = zi - zs;
        a_ii += -ppe_coefficient3(sc, lf, dsqrt_rn(dot3(ddx, ddy, ddz, ddx, ddy, ddz)));
    }
    st.ppe_col_tmp[ell(m, n, i)] = i;
    st.ppe_val_tmp[ell(m, n, i)] = a_ii;
    st.ppe_len[i] = m + 1;
}

// Detail::InvertMatrix<3> (Computer.hpp:364-422): the cofactor formula as written there
// (each minor placed at its own index), or val times the identity for a zero determinant.
// a is row-major.
__device__ __forceinline__ void gc_invert3(const double* a, double val, double* m) {
    const double a00 = a[0], a01 = a[1], a02 = a[2];
    const double a10 = a[3], a11 = a[4], a12 = a[5];
    const double a20 = a[6], a21 = a[7], a22 = a[8];
    double det = a00 * a11 * a22;
    det = det + a01 * a12 * a20;
    det = det + a02 * a10 * a21;
    det = det - a00 * a12 * a21;
    det = det - a01 * a10 * a22;
    det = det - a02 * a11 * a20;
    if (det == 0) {
        for (int k = 0; k < 9; k++) m[k] = (k % 4 == 0) ? val : 0.0;
        return;
    }
    auto d2 = [](double p, double q, double r, double s) { return p * s - q * r; };
    m[0] = d2(a11, a12, a21, a22) / det;
    m[1] = -d2(a10, a12, a20, a22) / det;
    m[2] = d2(a10, a11, a20, a21) / det;
    m[3] = -d2(a01, a02, a21, a22) / det;
    m[4] = d2(a00, a02, a20, a22) / det;
    m[5] = -d2(a00, a01, a20, a21) / det;
    m[6] = d2(a01, a02, a11, a12) / det;
    m[7] = -d2(a00, a02, a10, a12) / det;
    m[8] = d2(a00, a01, a10, a11) / det;
}

// uBLAS prod(C, dx), row k summed from 0
__device__ __forceinline__ double row3(const double* c, double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(c[0], dx)), __dmul_rn(c[1], dy)), __dmul_rn(c[2], dz));
}

// ModifyByPressureGradient (Computer.hpp:1433-1521): du only.  kGc: the corrective
// matrix (a first walk sums C^-1 = sum W / r^2 dx dx^T; the off-diagonal products are
// equal bit for bit, so one accumulator serves each pair).
template <bool kGc>
__global__ void k3_pressure_gradient(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    const double xi = st.x[i], yi = st.y[i], zi = st.z[i], pi = st.p[i];
    double gx = 0.0, gy = 0.0, gz = 0.0;
    double C[9];
    if (kGc) {
        double m00 = 0.0, m01 = 0.0, m02 = 0.0, m11 = 0.0, m12 = 0.0, m22 = 0.0;
        for_near3(sc, st, i, sc.f32_out_re, [&](int j) {
            const double dx = st.x[j] - xi;
            const double dy = st.y[j] - yi;
            const double dz = st.z[j] - zi;
            const double r2 = dist3(dx, dy, dz);
            if (!below(r2, sc.re2)) return;
            const double wg = weight(dsqrt_rn(r2), sc.re);
            const double t = ddiv_rn(wg, r2);
            m00 += t * (dx * dx);
            m01 += t * (dx * dy);
            m02 += t * (dx * dz);
            m11 += t * (dy * dy);
            m12 += t * (dy * dz);
            m22 += t * (dz * dz);
            if (spp) {
                gx += wg * dx;
                gy += wg * dy;
                gz += wg * dz;
            }
        });
        double xs, ys, zs;
        if (spp && spp_particle3(sc, st, i, sc.re, gx, gy, gz, xs, ys, zs)) {
            const double dx = xs - xi, dy = ys - yi, dz = zs - zi;
            const double r2 = dist3(dx, dy, dz);
            const double t = ddiv_rn(weight(dsqrt_rn(r2), sc.re), r2);
            m00 += t * (dx * dx);
            m01 += t * (dx * dy);
            m02 += t * (dx * dz);
            m11 += t * (dy * dy);
            m12 += t * (dy * dz);
            m22 += t * (dz * dz);
        }
        const double a[9] = {m00, m01, m02, m01, m11, m12, m02, m12, m22};
        gc_invert3(a, 3.0 / sc.n0, C);  // InvertMatrix(invC, DIM / n0)
        gx = gy = gz = 0.0;
    }
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for_near3(sc, st, i, sc.f32_out_re, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dy = st.y[j] - yi;
        const double dz = st.z[j] - zi;
        const double r2 = dist3(dx, dy, dz);
        if (!below(r2, sc.re2)) return;
        const double wg = weight(dsqrt_rn(r2), sc.re);
        if (st.type[j] != MPS_TYPE_DUMMY) {
            const double c = ddiv_rn(st.p[j] + pi, r2) * wg;
            if (kGc) {
                sx += c * row3(C, dx, dy, dz);
                sy += c * row3(C + 3, dx, dy, dz);
                sz += c * row3(C + 6, dx, dy, dz);
            } else {
                sx += c * dx;
                sy += c * dy;
                sz += c * dz;
            }
        }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        if (spp) {
            gx += wg * dx;
            gy += wg * dy;
            gz += wg * dz;
        }
    });
    double xs, ys, zs;
    if (spp && spp_particle3(sc, st, i, sc.re, gx, gy, gz, xs, ys, zs)) {
        const double dx = xs - xi, dy = ys - yi, dz = zs - zi;
        const double r2 = dist3(dx, dy, dz);
        const double c = ddiv_rn(0.0 + pi, r2) * weight(dsqrt_rn(r2), sc.re);
        if (kGc) {
            sx += c * row3(C, dx, dy, dz);
            sy += c * row3(C + 3, dx, dy, dz);
            sz += c * row3(C + 6, dx, dy, dz);
        } else {
            sx += c * dx;
            sy += c * dy;
            sz += c * dz;
        }
    }
    const double dt = st.step->dt;
    const double factor = kGc ? -dt * st.nd[i] / (sc.rho * sc.n0) : -dt / sc.rho * 3.0 / sc.n0;
    st.dux[i] = factor * sx;
    st.duy[i] = factor * sy;
    st.duz[i] = factor * sz;
}

// DynamicStabilize (Computer.hpp:1568-1635): du only.
__global__ void k3_dynamic_stabilize(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const double dt = st.step->dt;
    const double d = sc.l0 - sc.max_dx;
    const double d2 = d * d;
    const double factor = -1.0 / (2 * dt * sc.n0);
    const double xi = st.x[i], yi = st.y[i], zi = st.z[i];
    const double oxi = st.ox[i], oyi = st.oy[i], ozi = st.oz[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for_near3(sc, st, i, fminf(sc.f32_out_re, sc.f32_out_ds), [&](int j) {
        const double dx = st.x[j] - xi;
        const double dy = st.y[j] - yi;
        const double dz = st.z[j] - zi;
        const double r2 = dist3(dx, dy, dz);
        if (!below(r2, sc.re2)) return;
        if (st.type[j] != MPS_TYPE_DUMMY && below(r2, d2)) {
            const double dx0 = st.ox[j] - oxi;
            const double dy0 = st.oy[j] - oyi;
            const double dz0 = st.oz[j] - ozi;
            const double nrm = dsqrt_rn(dot3(dx0, dy0, dz0, dx0, dy0, dz0));
            const double ex = ddiv_rn(dx0, nrm), ey = ddiv_rn(dy0, nrm), ez = ddiv_rn(dz0, nrm);
            const double r_par = dot3(dx, dy, dz, ex, ey, ez);
            const double px = dx - r_par * ex;
            const double py = dy - r_par * ey;
            const double pz = dz - r_par * ez;
            const double r_perp2 = dot3(px, py, pz, px, py, pz);
            const double mag = dsqrt_rn(d2 - r_perp2) - r_par;
            sx += mag * ex;
            sy += mag * ey;
            sz += mag * ez;
        }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
    });
    // With SPP the reference places the virtual particle too but leaves it out of the sum
    // (Computer.hpp:1597-1598): a zero vector, so it is not built here.
    st.dux[i] = factor * sx;
    st.duy[i] = factor * sy;
    st.duz[i] = factor * sz;
}

// u += du; x += du dt for fluid particles (Computer.hpp:1543-1563, :1637-1655)
__global__ void k3_apply_du(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const double dt = st.step->dt;
    const double dx = st.dux[i], dy = st.duy[i], dz = st.duz[i];
    st.u[i] = st.u[i] + dx;
    st.v[i] = st.v[i] + dy;
    st.w[i] = st.w[i] + dz;
    st.x[i] = st.x[i] + dx * dt;
    st.y[i] = st.y[i] + dy * dt;
    st.z[i] = st.z[i] + dz * dt;
    positions_f32(st, i);
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_search3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_bucket<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    launch_cell_sort(sc, st, s);
    k3_neighbors<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_cfl_dt3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_max_speed<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    launch_cfl_dt_finish(sc, st, s);
}

void launch_density3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_density<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_error_correction3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_error_correction<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_density_variation3(const SceneConst& sc, const DeviceState& st, double* out, cudaStream_t s) {
    k3_density_variation<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st, out);
}

void launch_explicit3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_explicit_accel<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    k3_explicit_update<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_save_x3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_save_x<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_set_ppe3(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s) {
    k3_ppe_build<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    launch_ppe_layout(sc, st, want_fp32, s);
}

void launch_pressure_gradient3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    if (sc.flags & MPS_FLAG_GC)
        k3_pressure_gradient<true><<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    else
        k3_pressure_gradient<false><<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    k3_apply_du<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_dynamic_stabilize3(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k3_dynamic_stabilize<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    k3_apply_du<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

}  // namespace mpsgb
