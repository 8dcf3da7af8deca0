// stages.cu - the per-particle stages of Computer::ForwardTime (Computer.hpp:1700-1742):
// number density, error-compensating source, explicit forces, PPE right-hand side and
// matrix assembly, pressure assignment (or the explicit pressure), midpoint pressure
// gradient (plain or with the GC corrective matrix), dynamic stabilisation and the CFL
// time step.
//
// One thread per particle walks its neighbour row in reference order and accumulates
// exactly like AccumulateNeighbor (Computer.hpp:618-695): the filter r^2 < r_e^2 on
// current positions, the terms in list order, the SPP virtual particle last.  The
// filter runs in two steps (for_near): an FP32 screen that drops entries surely out of
// range, then the reference's FP64 test on the rest, which decides as before.  Every
// formula keeps the reference's expression order and this file is compiled with
// -fmad=false, so each result is bit-identical to the FP64 CPU path.
#include "common.cuh"

namespace mpsgb {

namespace {

__device__ __forceinline__ bool is_surface(const SceneConst& sc, double nd) {
    return ddiv_rn(nd, sc.n0) < sc.surface_ratio;  // Computer.hpp:586-589
}

// The SPP virtual particle of AccumulateNeighbor (Computer.hpp:664-692).  (gx, gz)
// holds sum W(r) dx over the neighbours within `radius`.
__device__ __forceinline__ bool spp_particle(const SceneConst& sc, const DeviceState& st, int i,
                                             double radius, double gx, double gz, double& xs,
                                             double& zs) {
    const double thisN = st.n_wo_spp[i];
    gx = ddiv_rn(gx, sc.n0);
    gz = ddiv_rn(gz, sc.n0);
    if (thisN < sc.n0) {
        const double r_g = dsqrt_rn(dot2(gx, gz, gx, gz));
        if (r_g > 2.220446049250313080847e-16) {  // std::numeric_limits<double>::epsilon()
            const double w_spp = __dadd_rn(sc.n0, -thisN);
            const double r_spp = ddiv_rn(radius, __dadd_rn(w_spp, 1.0));
            const double s = ddiv_rn(r_spp, r_g);
            xs = __dadd_rn(st.x[i], -__dmul_rn(s, gx));
            zs = __dadd_rn(st.z[i], -__dmul_rn(s, gz));
            return true;
        }
    }
    return false;
}

// a = viscosity + G (Computer.hpp:980-988): G = (0, -g), or with MPS_FLAG_CENTRAL_GRAVITY
// G_z c with c = x / |x|, c = 0 within l0 / 100 of the origin.
__device__ __forceinline__ void add_gravity(const SceneConst& sc, double xi, double zi, double vx, double vz,
                                            double& ax, double& az) {
    if (has_flag(sc.flags, MPS_FLAG_CENTRAL_GRAVITY)) {
        const double g = -sc.g;
        const double r = dsqrt_rn(dot2(xi, zi, xi, zi));
        double cx = 0.0, cz = 0.0;
        if (!(r < sc.l0 * 0.01)) {
            cx = xi / r;
            cz = zi / r;
        }
        ax = vx + g * cx;
        az = vz + g * cz;
    } else {
        ax = __dadd_rn(vx, 0.0);
        az = vz + (-sc.g);
    }
}

// NeighborDensityVariationSpeed (Computer.hpp:838-872)
__device__ double density_variation(const SceneConst& sc, const DeviceState& st, int i,
                                    double dt) {
    if (has_flag(sc.flags, MPS_FLAG_HS)) {
        if (has_flag(sc.flags, MPS_FLAG_SPP) && st.n_wo_spp[i] < sc.n0) return 0.0;
        const double xi = st.x[i], zi = st.z[i], ui = st.u[i], wi = st.w[i];
        double sum = 0.0;
        for_near(sc, st, i, sc.f32_out_re, [&](int j) {
            const double dx = st.x[j] - xi;
            const double dz = st.z[j] - zi;
            const double r2 = dist2(dx, dz);
            if (below(r2, sc.re2)) {
                const double du = st.u[j] - ui;
                const double dw = st.w[j] - wi;
                const double r = dsqrt_rn(r2);
                sum += ddiv_rn(dot2_term(dx, dz, du, dw), r * r * r);
            }
        });
        return -sc.re * sum;
    }
    return (st.nd[i] - sc.n0) / dt;
}

// The constant factors of the Laplacian coefficients, evaluated once per thread in the
// reference's left-to-right order (so each coefficient is the same rounding chain).
struct LapFactors {
    bool hl;
    double visc;  // HL: ((nu 3) re_lap) / n0_lap; else (((nu 2) 2) / lambda_lap) / n0_lap
    double ppe;   // HL: (3 re_lap) / n0_lap;       else (4 / lambda_lap) / n0_lap
};
__device__ __forceinline__ LapFactors lap_factors(const SceneConst& sc) {
    LapFactors f;
    f.hl = has_flag(sc.flags, MPS_FLAG_HL);
    f.visc = f.hl ? sc.nu * 3.0 * sc.re_lap / sc.n0_lap : sc.nu * 2 * 2.0 / sc.lambda_lap / sc.n0_lap;
    f.ppe = f.hl ? 3.0 * sc.re_lap / sc.n0_lap : 4.0 / sc.lambda_lap / sc.n0_lap;
    return f;
}

// viscosity coefficient (Computer.hpp:963-970) at the Laplacian radius
__device__ __forceinline__ double viscosity_coefficient(const SceneConst& sc, const LapFactors& f, double r) {
    if (f.hl) return ddiv_rn(f.visc, r * r * r);
    return f.visc * weight(r, sc.re_lap);
}

// PPE off-diagonal coefficient (Computer.hpp:1290-1297)
__device__ __forceinline__ double ppe_coefficient(const SceneConst& sc, const LapFactors& f, double r) {
    if (f.hl) return ddiv_rn(f.ppe, r * r * r);
    return f.ppe * weight(r, sc.re_lap);
}

__device__ __forceinline__ bool ppe_alive(const SceneConst& sc, const DeviceState& st, int i) {
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return false;
    if (!has_flag(sc.flags, MPS_FLAG_SPP) && is_surface(sc, st.nd[i])) return false;
    return true;
}

// ------------------------------------------------------------------ kernels
__global__ void k_set_dt(DeviceState st, double dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st.step->dt = dt;  // Computer.hpp:1703-1706
        st.step->t = st.step->t + dt;
    }
}

// DetermineDt (Computer.hpp:759-777), part 1: max |u|^2 over all particles.
__global__ void k_max_speed(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < sc.n) v = dot2(st.u[i], st.w[i], st.u[i], st.w[i]);
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0)
        atomicMax(&st.step->max_u2_bits, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// part 2: dt = maxU == 0 ? MaxDt : min(MaxDx / maxU, MaxDt); then t += dt.
__global__ void k_cfl_dt(SceneConst sc, DeviceState st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double u2 = __longlong_as_double(static_cast<long long>(st.step->max_u2_bits));
        const double maxU = dsqrt_rn(u2);
        double dt;
        if (maxU == 0) {
            dt = sc.max_dt;
        } else {
            const double a = sc.max_dx / maxU;
            dt = (sc.max_dt < a) ? sc.max_dt : a;
        }
        st.step->dt = dt;
        st.step->t = st.step->t + dt;
        st.step->max_u2_bits = 0ull;
    }
}

// ComputeNeighborDensities (Computer.hpp:780-833)
__global__ void k_density(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    if (spp) st.n_wo_spp[i] = sc.n0;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const double xi = st.x[i], zi = st.z[i];
    double thisN = 0.0;
    for_near(sc, st, i, sc.f32_out_re, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.re2)) thisN += weight(dsqrt_rn(r2), sc.re);
    });
    if (spp) {
        st.n_wo_spp[i] = thisN;
        st.nd[i] = (thisN < sc.n0) ? sc.n0 : thisN;  // std::max(thisN, n0)
    } else {
        st.nd[i] = thisN;
    }
}

// With PRESSURE_EXPLICIT: the second ComputeNeighborDensities and the pressure of
// ComputeImplicitForces (Computer.hpp:1046-1067) in one pass.  The pressure reads only
// the particle's own density, and SaveX between the two stages touches neither, so the
// results equal the separate kernels.  W(r, r_e) of the entries in range is cached for
// the pressure gradient (same positions, same list order), as k_density_ppe does.
__global__ void k_density_explicit_pressure(SceneConst sc, DeviceState st, int32_t* ok) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && ok) *ok = 1;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    if (spp) st.n_wo_spp[i] = sc.n0;
    const int t = st.type[i];
    double nd = st.nd[i];  // dummy and disabled particles keep theirs
    if (t != MPS_TYPE_DUMMY && t != MPS_TYPE_DISABLED) {
        const int n = sc.n;
        const double xi = st.x[i], zi = st.z[i];
        double thisN = 0.0;
        int m_re = 0;
        for_near(sc, st, i, sc.f32_out_re, [&](int j) {
            const double dx = st.x[j] - xi;
            const double dz = st.z[j] - zi;
            const double r2 = dist2(dx, dz);
            if (below(r2, sc.re2)) {
                const double w = weight(dsqrt_rn(r2), sc.re);
                thisN += w;
                if (m_re < kReCache) st.w_re[static_cast<int64_t>(m_re) * n + i] = w;
                m_re++;
            }
        });
        if (spp) {
            st.n_wo_spp[i] = thisN;
            nd = (thisN < sc.n0) ? sc.n0 : thisN;
        } else {
            nd = thisN;
        }
        st.nd[i] = nd;
    }
    const double rho0 = sc.rho;
    const double c = sc.sound_speed;
    const double rho = rho0 / sc.n0 * nd;
    st.p[i] = (rho <= rho0) ? 0.0 : c * c * (rho - rho0);
}

// ComputeErrorCorrection (Computer.hpp:877-910)
__global__ void k_error_correction(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const double speed = density_variation(sc, st, i, st.step->dt);
    const double error = (st.nd[i] - sc.n0) / sc.n0;
    st.ecs[i] = fabs(error) * speed + fabs(speed) * error;
}

__global__ void k_density_variation(SceneConst sc, DeviceState st, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    const int t = st.type[i];
    out[i] = (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED)
                 ? 0.0
                 : density_variation(sc, st, i, st.step->dt);
}

// ComputeExplicitForces, first loop (Computer.hpp:935-990): a = viscosity + g.
__global__ void k_explicit_accel(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const LapFactors lf = lap_factors(sc);
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const double xi = st.x[i], zi = st.z[i], ui = st.u[i], wi = st.w[i];
    double vx = 0.0, vz = 0.0;
    for_near(sc, st, i, sc.f32_out_rl, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.rl2)) {
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double c = viscosity_coefficient(sc, lf, dsqrt_rn(r2));
                vx += c * (st.u[j] - ui);
                vz += c * (st.w[j] - wi);
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        }
    });
    // With SPP the reference adds the virtual particle's viscosity term c (u_i - u_i),
    // which is +0 for finite velocities: the virtual particle is not built here
    // (sums_from_zero, common.cuh).
    add_gravity(sc, xi, zi, vx, vz, st.dux[i], st.duz[i]);  // a += G (Environment.hpp:149)
}

// The stages between the search and the move in one walk over each neighbour row:
// ComputeNeighborDensities, ComputeErrorCorrection (with ECS) and the first loop of
// ComputeExplicitForces (fluid particles).  All three read positions and velocities that
// none of them writes, and each writes only its own particle's results, so one walk
// gives exactly what k_density, k_error_correction and k_explicit_accel give: every
// accumulator sees the same terms in the same list order, and the square root of a pair
// is computed once for all of them.
template <bool kEcs>
__global__ void k_pre_pressure(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const LapFactors lf = lap_factors(sc);
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    if (spp) st.n_wo_spp[i] = sc.n0;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const bool fluid = t == MPS_TYPE_FLUID;
    const bool hs = kEcs && has_flag(sc.flags, MPS_FLAG_HS);
    const double xi = st.x[i], zi = st.z[i], ui = st.u[i], wi = st.w[i];
    double thisN = 0.0, hsum = 0.0;
    double vx = 0.0, vz = 0.0;
    const float out_thr = fluid ? fmaxf(sc.f32_out_re, sc.f32_out_rl) : sc.f32_out_re;
    for_near(sc, st, i, out_thr, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        const bool in_re = below(r2, sc.re2);
        const bool in_rl = fluid && below(r2, sc.rl2);
        if (!in_re && !in_rl) return;
        const double r = dsqrt_rn(r2);
        if (in_re) {
            thisN += weight(r, sc.re);
            if (hs) {
                const double du = st.u[j] - ui;
                const double dw = st.w[j] - wi;
                hsum += ddiv_rn(dot2_term(dx, dz, du, dw), r * r * r);
            }
        }
        if (in_rl) {
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double c = viscosity_coefficient(sc, lf, r);
                vx += c * (st.u[j] - ui);
                vz += c * (st.w[j] - wi);
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        }
    });
    // ComputeNeighborDensities
    double nd;
    if (spp) {
        st.n_wo_spp[i] = thisN;
        nd = (thisN < sc.n0) ? sc.n0 : thisN;
    } else {
        nd = thisN;
    }
    st.nd[i] = nd;
    // ComputeErrorCorrection (NeighborDensityVariationSpeed on the same walk)
    if (kEcs) {
        double speed;
        if (has_flag(sc.flags, MPS_FLAG_HS)) {
            speed = (spp && thisN < sc.n0) ? 0.0 : -sc.re * hsum;
        } else {
            speed = (nd - sc.n0) / st.step->dt;
        }
        const double error = (nd - sc.n0) / sc.n0;
        st.ecs[i] = fabs(error) * speed + fabs(speed) * error;
    }
    if (!fluid) return;
    // ComputeExplicitForces, first loop
    // With SPP the reference adds the virtual particle's viscosity term c (u_i - u_i),
    // which is +0 for finite velocities: the virtual particle is not built here
    // (sums_from_zero, common.cuh).
    add_gravity(sc, xi, zi, vx, vz, st.dux[i], st.duz[i]);
}

// ComputeExplicitForces, second loop (Computer.hpp:995-1020).
__global__ void k_explicit_update(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const double dt = st.step->dt;
    if (st.type[i] == MPS_TYPE_FLUID) {
        const double u = st.u[i] + st.dux[i] * dt;
        const double w = st.w[i] + st.duz[i] * dt;
        st.u[i] = u;
        st.w[i] = w;
        const double x = st.x[i] + u * dt;
        const double z = st.z[i] + w * dt;
        st.x[i] = x;
        st.z[i] = z;
        st.x32[i] = __double2float_rn(x);
        st.z32[i] = __double2float_rn(z);
    } else {
        const double nx = st.wall_x[i], nz = st.wall_z[i];
        st.u[i] = (nx - st.x[i]) / dt;
        st.w[i] = (nz - st.z[i]) / dt;
        st.x[i] = nx;
        st.z[i] = nz;
        st.x32[i] = __double2float_rn(nx);
        st.z32[i] = __double2float_rn(nz);
    }
}

// SaveX (Computer.hpp:1025-1039)
__global__ void k_save_x(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    st.ox[i] = st.x[i];
    st.oz[i] = st.z[i];
}

// One PPE row as the assembly walk produces it: its off-diagonal entries in neighbour
// order, then the diagonal.  With the ELL scratch, entry m of particle i goes to
// [m n + i] and k_ppe_sort orders the row later.  In direct mode (rows in cell order)
// the columns arrive ascending: the neighbour list walks the cells in ascending index and
// each cell in row order.  So entry m goes straight to its rank among the row's SELL
// slots (m before the diagonal, m + 1 after it) and the diagonal to the count of columns
// below it: the ascending-column layout of the reference's compressed matrix
// (Computer.hpp:1330-1350).  A column out of order fails the step (it cannot happen for
// cell-ordered rows).
struct PpeRow {
    int i, row, m, below, prev;
    __device__ PpeRow(int i_, int row_) : i(i_), row(row_), m(0), below(0), prev(-1) {}
    __device__ __forceinline__ void store(const SceneConst& sc, const DeviceState& st, int rank, int col,
                                          double v) const {
        const int64_t base = static_cast<int64_t>(row / kSellRows) * sc.ppe_stride * kSellRows;
        const int64_t at = sell_index(base, row % kSellRows, rank);
        st.ppe_col[at] = col;
        st.ppe_val[at] = v;
        if (st.ppe_fp32) st.ppe_cv32[at] = make_uint2(static_cast<unsigned>(col), __float_as_uint(__double2float_rn(v)));
    }
    __device__ __forceinline__ void put(const SceneConst& sc, const DeviceState& st, int col, double v) {
        if (st.ppe_direct) {
            if (col <= prev) {
                atomicOr(&st.status->flags, kStatusDeviceCheck);
                st.status->check_index = i;
            }
            prev = col;
            below += col < row ? 1 : 0;
            store(sc, st, m + (col > row ? 1 : 0), col, v);
        } else {
            st.ppe_col_tmp[ell(m, sc.n, i)] = col;
            st.ppe_val_tmp[ell(m, sc.n, i)] = v;
        }
        m++;
    }
    __device__ __forceinline__ void diag(const SceneConst& sc, const DeviceState& st, double a_ii) {
        if (st.ppe_direct) {
            store(sc, st, below, row, a_ii);
        } else {
            st.ppe_col_tmp[ell(m, sc.n, i)] = row;
            st.ppe_val_tmp[ell(m, sc.n, i)] = a_ii;
        }
        st.ppe_len[row] = m + 1;
    }
};

// SetPressurePoissonEquation (Computer.hpp:1145-1328): right-hand side, initial guess
// and one matrix row per particle in neighbour order (diagonal last) into the
// scratch ELL arrays (column k of particle i at [k n + i]).  Rows and columns are PPE
// rows (ppe_row); b, x and the row length are stored at the particle's row.
__global__ void k_ppe_build(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const LapFactors lf = lap_factors(sc);
    const int row = ppe_row(st, i);
    if (!ppe_alive(sc, st, i)) {
        st.ppe_b[row] = 0;
        st.ppe_x[row] = 0;
        PpeRow(i, row).diag(sc, st, 1.0);
        return;
    }
    const double dt = st.step->dt;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    const double speed = density_variation(sc, st, i, dt);
    if (has_flag(sc.flags, MPS_FLAG_ECS)) {
        const double e = st.ecs[i];
        st.ppe_b[row] = -sc.rho / (sc.n0 * dt) * (speed + e);
    } else {
        st.ppe_b[row] = -sc.rho / (sc.n0 * dt) * speed;
    }
    st.ppe_x[row] = st.p[i];

    const double xi = st.x[i], zi = st.z[i];
    double a_ii = 0.0, gx = 0.0, gz = 0.0;
    PpeRow pr(i, row);
    for_near(sc, st, i, sc.f32_out_rl, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.rl2)) {
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double a_ij = ppe_coefficient(sc, lf, dsqrt_rn(r2));
                if (spp || !is_surface(sc, st.nd[j])) pr.put(sc, st, ppe_row(st, j), a_ij);
                a_ii += -a_ij;
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
            if (spp) {
                const double wg = weight(dsqrt_rn(r2), sc.re_lap);
                gx += wg * dx;
                gz += wg * dz;
            }
        }
    });
    double xs, zs;
    if (spp && spp_particle(sc, st, i, sc.re_lap, gx, gz, xs, zs)) {
        const double ddx = xi - xs, ddz = zi - zs;
        a_ii += -ppe_coefficient(sc, lf, dsqrt_rn(dot2(ddx, ddz, ddx, ddz)));
    }
    pr.diag(sc, st, a_ii);
}

// Number density after the move (the second ComputeNeighborDensities) and the PPE
// assembly in one walk over each neighbour row, for the SPP method set: there the
// assembly reads only the particle's own density (space potential particles replace the
// surface test on the neighbours' densities), so the two stages fuse.  The density and
// source terms run on the entries within r_e, the Laplacian on those within the
// Laplacian radius, each in list order as in k_density and k_ppe_build.
__global__ void k_density_ppe(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const LapFactors lf = lap_factors(sc);
    const int n = sc.n;
    const int row = ppe_row(st, i);
    st.n_wo_spp[i] = sc.n0;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) {
        st.ppe_b[row] = 0;
        st.ppe_x[row] = 0;
        PpeRow(i, row).diag(sc, st, 1.0);
        return;
    }
    const bool hs = has_flag(sc.flags, MPS_FLAG_HS);
    const double xi = st.x[i], zi = st.z[i], ui = st.u[i], wi = st.w[i];
    double thisN = 0.0, hsum = 0.0, a_ii = 0.0, gx = 0.0, gz = 0.0;
    int m_re = 0;
    PpeRow pr(i, row);
    for_near(sc, st, i, fmaxf(sc.f32_out_re, sc.f32_out_rl), [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        const bool in_re = below(r2, sc.re2);
        const bool in_rl = below(r2, sc.rl2);
        if (!in_re && !in_rl) return;
        const double r = dsqrt_rn(r2);
        // W(r, r_e), reused for W(r, r_e^lap) when the two radii are one
        const double w = in_re ? weight(r, sc.re) : 0.0;
        if (in_re) {
            thisN += w;
            if (m_re < kReCache) st.w_re[static_cast<int64_t>(m_re) * n + i] = w;
            m_re++;
            if (hs) {
                const double du = st.u[j] - ui;
                const double dw = st.w[j] - wi;
                hsum += ddiv_rn(dot2_term(dx, dz, du, dw), r * r * r);
            }
        }
        if (in_rl) {
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double a_ij = ppe_coefficient(sc, lf, r);
                pr.put(sc, st, ppe_row(st, j), a_ij);
                a_ii += -a_ij;
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
            const double wg = (in_re && sc.re_lap == sc.re) ? w : weight(r, sc.re_lap);
            gx += wg * dx;
            gz += wg * dz;
        }
    });
    // ComputeNeighborDensities
    st.n_wo_spp[i] = thisN;
    const double nd = (thisN < sc.n0) ? sc.n0 : thisN;
    st.nd[i] = nd;
    // right-hand side (NeighborDensityVariationSpeed) and initial guess
    const double dt = st.step->dt;
    const double speed = hs ? ((thisN < sc.n0) ? 0.0 : -sc.re * hsum) : (nd - sc.n0) / dt;
    if (has_flag(sc.flags, MPS_FLAG_ECS)) {
        const double e = st.ecs[i];
        st.ppe_b[row] = -sc.rho / (sc.n0 * dt) * (speed + e);
    } else {
        st.ppe_b[row] = -sc.rho / (sc.n0 * dt) * speed;
    }
    st.ppe_x[row] = st.p[i];
    st.spp_g[i] = gx;
    st.spp_g[n + i] = gz;
    double xs, zs;
    if (spp_particle(sc, st, i, sc.re_lap, gx, gz, xs, zs)) {
        const double ddx = xi - xs, ddz = zi - zs;
        a_ii += -ppe_coefficient(sc, lf, dsqrt_rn(dot2(ddx, ddz, ddx, ddz)));
    }
    pr.diag(sc, st, a_ii);
}

// Chunk sizes of the SELL-32 layout: one warp per chunk of 32 rows.
__global__ void k_ppe_chunks(SceneConst sc, DeviceState st) {
    const int c = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (c >= sc.nchunks) return;
    if (step_failed(sc, st)) return;
    const int lane = threadIdx.x & 31;
    const int len = st.ppe_len[c * kSellRows + lane];
    warp_add_u64(&st.status->ppe_nnz, static_cast<unsigned long long>(len));
    const int m = __reduce_max_sync(0xffffffffu, len);
    if (lane == 0) st.ppe_chunk[c] = static_cast<int>(sell_chunk_size(m));
}

// Row entries to ascending column order (uBLAS compressed_matrix, Computer.hpp:1330-1350):
// each entry goes to its rank among the row's columns (columns are distinct), at its
// SELL-32 position.  One thread per particle (coalesced scratch reads), writing its row.
__global__ void k_ppe_sort(SceneConst sc, DeviceState st, int want_fp32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (step_failed(sc, st)) return;
    const int n = sc.n;
    if (i >= n) return;
    const int row = ppe_row(st, i);
    const int len = st.ppe_len[row];
    const int64_t base = st.ppe_off[row / kSellRows];
    const int r = row % kSellRows;
    auto put = [&](int e, int rank) {
        const int ce = st.ppe_col_tmp[ell(e, n, i)];
        const double v = st.ppe_val_tmp[ell(e, n, i)];
        const int64_t at = sell_index(base, r, rank);
        st.ppe_col[at] = ce;
        st.ppe_val[at] = v;
        if (want_fp32) st.ppe_cv32[at] = make_uint2(static_cast<unsigned>(ce),
                                                     __float_as_uint(__double2float_rn(v)));
    };
    // Rows in search-cell order: a neighbour list walks the cells in ascending cell index
    // and each cell in slot (= row) order, so the off-diagonal columns arrive ascending and
    // only the diagonal (last) needs its place.  Checked on the way; a row that is not
    // ascending takes the general rank computation.
    bool ascending = st.row_of != nullptr;
    for (int e = 1; ascending && e < len - 1; e++)
        ascending = st.ppe_col_tmp[ell(e - 1, n, i)] < st.ppe_col_tmp[ell(e, n, i)];
    if (ascending) {
        int below_diag = 0;
        for (int e = 0; e < len - 1; e++) {
            const bool after = st.ppe_col_tmp[ell(e, n, i)] > row;
            below_diag += after ? 0 : 1;
            put(e, e + (after ? 1 : 0));
        }
        put(len - 1, below_diag);
        return;
    }
    for (int e = 0; e < len; e++) {
        const int ce = st.ppe_col_tmp[ell(e, n, i)];
        int rank = 0;
        for (int f = 0; f < len; f++) rank += (st.ppe_col_tmp[ell(f, n, i)] < ce) ? 1 : 0;
        put(e, rank);
    }
}

// ComputeImplicitForces pressure assignment (Computer.hpp:1076-1097)
__global__ void k_assign_pressure(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    const int t = st.type[i];
    if (t == MPS_TYPE_DUMMY || t == MPS_TYPE_DISABLED) return;
    const double v = st.ppe_x[ppe_row(st, i)];
    const bool surface = !has_flag(sc.flags, MPS_FLAG_SPP) && is_surface(sc, st.nd[i]);
    st.p[i] = ((v < 0) || surface) ? 0.0 : v;
}

// ModifyByPressureGradient, midpoint branch (Computer.hpp:1501-1521): du only.
// kCache >= 1: W of the entries within r_e comes from st.w_re (the density walk wrote it
// on the same positions, in the same list order); 2: the SPP sums come from st.spp_g too.
template <int kCache>
__global__ void k_pressure_gradient(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    const double dt = st.step->dt;
    const double factor = -dt / sc.rho * 2.0 / sc.n0;
    const double xi = st.x[i], zi = st.z[i], pi = st.p[i];
    double sx = 0.0, sz = 0.0, gx = 0.0, gz = 0.0;
    int m_re = 0;
    for_near(sc, st, i, sc.f32_out_re, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.re2)) {
            const double wg = (kCache >= 1 && m_re < kReCache) ? st.w_re[static_cast<int64_t>(m_re) * sc.n + i]
                                                               : weight(dsqrt_rn(r2), sc.re);
            m_re++;
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double c = ddiv_rn(st.p[j] + pi, r2) * wg;
                sx += c * dx;
                sz += c * dz;
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
            if (kCache < 2 && spp) {
                gx += wg * dx;
                gz += wg * dz;
            }
        }
    });
    if (kCache == 2 && spp) {
        gx = st.spp_g[i];
        gz = st.spp_g[sc.n + i];
    }
    double xs, zs;
    if (spp && spp_particle(sc, st, i, sc.re, gx, gz, xs, zs)) {
        const double dx = xs - xi;
        const double dz = zs - zi;
        const double r2 = dist2(dx, dz);
        const double c = ddiv_rn(0.0 + pi, r2) * weight(dsqrt_rn(r2), sc.re);
        sx += c * dx;
        sz += c * dz;
    }
    st.dux[i] = factor * sx;
    st.duz[i] = factor * sz;
}

// ComputeImplicitForces with PRESSURE_EXPLICIT (Computer.hpp:1046-1067): the virtual
// density rho0 / n0 n of every particle (dummy and disabled ones included, from the
// number density they carry) and p = c^2 (rho - rho0) above rho0, else 0.
__global__ void k_explicit_pressure(SceneConst sc, DeviceState st, int32_t* ok) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && ok) *ok = 1;
    if (i >= sc.n) return;
    if (step_failed(sc, st)) return;
    const double rho0 = sc.rho;
    const double c = sc.sound_speed;
    const double rho = rho0 / sc.n0 * st.nd[i];
    st.p[i] = (rho <= rho0) ? 0.0 : c * c * (rho - rho0);
}

// Detail::InvertMatrix<2> (Computer.hpp:323-347): the inverse of [[a, b], [b, d]], or
// val times the identity when the determinant is exactly zero.
__device__ __forceinline__ void gc_invert(double a, double b, double d, double val, double* m) {
    const double det = a * d - b * b;
    if (det == 0) {
        m[0] = val;
        m[1] = 0.0;
        m[2] = 0.0;
        m[3] = val;
        return;
    }
    m[0] = d / det;
    m[1] = -b / det;
    m[2] = -b / det;
    m[3] = a / det;
}

// prod(C, dx) of uBLAS: each row summed from 0 (0 + c0 dx) + c1 dz.
__device__ __forceinline__ double row_dot(double c0, double c1, double dx, double dz) {
    return __dadd_rn(__dadd_rn(0.0, __dmul_rn(c0, dx)), __dmul_rn(c1, dz));
}

// ModifyByPressureGradient with MPS_GC (Computer.hpp:1457-1499): du only.  The first
// walk sums C^-1 = sum W / r^2 dx dx^T over every neighbour within r_e and the SPP
// particle; the second sums (p_ij / r^2 W) C dx over the non-dummy ones in the same
// order.  The two off-diagonal sums of C^-1 add the same products (dx dz = dz dx
// exactly), so one accumulator holds both.
template <int kCache>
__global__ void k_pressure_gradient_gc(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const bool spp = has_flag(sc.flags, MPS_FLAG_SPP);
    const double xi = st.x[i], zi = st.z[i], pi = st.p[i];
    auto w_of = [&](int m, double r2) {
        return (kCache >= 1 && m < kReCache) ? st.w_re[static_cast<int64_t>(m) * sc.n + i]
                                             : weight(dsqrt_rn(r2), sc.re);
    };
    double m00 = 0.0, m01 = 0.0, m11 = 0.0, gx = 0.0, gz = 0.0;
    int m_re = 0;
    for_near(sc, st, i, sc.f32_out_re, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.re2)) {
            const double wg = w_of(m_re, r2);
            m_re++;
            const double t = ddiv_rn(wg, r2);
            m00 += t * (dx * dx);
            m01 += t * (dx * dz);
            m11 += t * (dz * dz);
            if (kCache < 2 && spp) {
                gx += wg * dx;
                gz += wg * dz;
            }
        }
    });
    if (kCache == 2 && spp) {  // the SPP sums of the density walk (see k_pressure_gradient)
        gx = st.spp_g[i];
        gz = st.spp_g[sc.n + i];
    }
    double xs = 0.0, zs = 0.0;
    const bool has_spp = spp && spp_particle(sc, st, i, sc.re, gx, gz, xs, zs);
    double sdx = 0.0, sdz = 0.0, sr2 = 0.0, sw = 0.0;
    if (has_spp) {
        sdx = xs - xi;
        sdz = zs - zi;
        sr2 = dist2(sdx, sdz);
        sw = weight(dsqrt_rn(sr2), sc.re);
        const double t = ddiv_rn(sw, sr2);
        m00 += t * (sdx * sdx);
        m01 += t * (sdx * sdz);
        m11 += t * (sdz * sdz);
    }
    double C[4];
    gc_invert(m00, m01, m11, 2.0 / sc.n0, C);  // InvertMatrix(invC, DIM / n0)
    double sx = 0.0, sz = 0.0;
    m_re = 0;
    for_near(sc, st, i, sc.f32_out_re, [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.re2)) {
            const double wg = w_of(m_re, r2);
            m_re++;
            if (st.type[j] != MPS_TYPE_DUMMY) {
                const double c = ddiv_rn(st.p[j] + pi, r2) * wg;
                sx += c * row_dot(C[0], C[1], dx, dz);
                sz += c * row_dot(C[2], C[3], dx, dz);
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        }
    });
    if (has_spp) {
        const double c = ddiv_rn(0.0 + pi, sr2) * sw;
        sx += c * row_dot(C[0], C[1], sdx, sdz);
        sz += c * row_dot(C[2], C[3], sdx, sdz);
    }
    const double dt = st.step->dt;
    const double factor = -dt * st.nd[i] / (sc.rho * sc.n0);
    st.dux[i] = factor * sx;
    st.duz[i] = factor * sz;
}

// DynamicStabilize (Computer.hpp:1568-1635): du only.
__global__ void k_dynamic_stabilize(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const double dt = st.step->dt;
    const double d = sc.l0 - sc.max_dx;
    const double d2 = d * d;
    const double factor = -1.0 / (2 * dt * sc.n0);
    const double xi = st.x[i], zi = st.z[i], oxi = st.ox[i], ozi = st.oz[i];
    double sx = 0.0, sz = 0.0;
    for_near(sc, st, i, fminf(sc.f32_out_re, sc.f32_out_ds), [&](int j) {
        const double dx = st.x[j] - xi;
        const double dz = st.z[j] - zi;
        const double r2 = dist2(dx, dz);
        if (below(r2, sc.re2)) {
            if (st.type[j] != MPS_TYPE_DUMMY && below(r2, d2)) {
                const double dx0 = st.ox[j] - oxi;
                const double dz0 = st.oz[j] - ozi;
                const double nrm = dsqrt_rn(dot2(dx0, dz0, dx0, dz0));
                const double ex = ddiv_rn(dx0, nrm);
                const double ez = ddiv_rn(dz0, nrm);
                const double r_par = dot2(dx, dz, ex, ez);
                const double px = dx - r_par * ex;
                const double pz = dz - r_par * ez;
                const double r_perp2 = dot2(px, pz, px, pz);
                const double mag = dsqrt_rn(d2 - r_perp2) - r_par;
                sx += mag * ex;
                sz += mag * ez;
            }  // the reference adds zero here: the identity on this sum (sums_from_zero, common.cuh)
        }
    });
    // With SPP the reference places the virtual particle too but leaves it out of the sum
    // (Computer.hpp:1597-1598): a zero vector, so it is not built here, and only pairs
    // within the collision distance d add anything: the FP32 screen uses the smaller of
    // d and r_e.
    st.dux[i] = factor * sx;
    st.duz[i] = factor * sz;
}

// u += du; x += du dt for fluid particles (Computer.hpp:1543-1563, :1637-1655)
__global__ void k_apply_du(SceneConst sc, DeviceState st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sc.n) return;
    if (solve_failed(sc, st)) return;
    if (st.type[i] != MPS_TYPE_FLUID) return;
    const double dt = st.step->dt;
    const double dx = st.dux[i], dz = st.duz[i];
    st.u[i] = st.u[i] + dx;
    st.w[i] = st.w[i] + dz;
    const double x = st.x[i] + dx * dt;
    const double z = st.z[i] + dz * dt;
    st.x[i] = x;
    st.z[i] = z;
    st.x32[i] = __double2float_rn(x);
    st.z32[i] = __double2float_rn(z);
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_set_dt(const SceneConst&, const DeviceState& st, double dt, cudaStream_t s) {
    k_set_dt<<<1, 32, 0, s>>>(st, dt);
}

void launch_cfl_dt(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_max_speed<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
    k_cfl_dt<<<1, 32, 0, s>>>(sc, st);
}

void launch_cfl_dt_finish(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_cfl_dt<<<1, 32, 0, s>>>(sc, st);
}

void launch_density(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_density<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
}

void launch_error_correction(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_error_correction<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
}

void launch_density_variation(const SceneConst& sc, const DeviceState& st, double* out,
                              cudaStream_t s) {
    k_density_variation<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st, out);
}

void launch_pre_pressure(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    if ((sc.flags & MPS_FLAG_ECS) != 0u)
        k_pre_pressure<true><<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
    else
        k_pre_pressure<false><<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
}

void launch_explicit_update(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_explicit_update<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_explicit(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_explicit_accel<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
    k_explicit_update<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_save_x(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_save_x<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

// Chunk widths (and the nonzero count); with the ELL scratch also the chunk offsets and
// the sorted rows.  Direct-mode rows are already in place, at fixed chunk offsets.
void launch_ppe_layout(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s) {
    k_ppe_chunks<<<grid_for(static_cast<int64_t>(sc.nchunks) * 32), kBlock, 0, s>>>(sc, st);
    if (st.ppe_direct) return;
    launch_exclusive_scan(st.ppe_chunk, st.ppe_off, sc.nchunks, st.scan_scratch, s);
    k_ppe_sort<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st, want_fp32 ? 1 : 0);
}

int set_ppe_launches(const DeviceState& st) { return st.ppe_direct ? 2 : kLaunchesSetPpe; }

// the state the assembly walk writes with: the FP32 copy of the matrix only when asked
DeviceState assembly_state(const DeviceState& st, bool want_fp32) {
    DeviceState a = st;
    a.ppe_fp32 = want_fp32 ? 1 : 0;
    return a;
}

void launch_set_ppe(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s) {
    k_ppe_build<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, assembly_state(st, want_fp32));
    launch_ppe_layout(sc, st, want_fp32, s);
}

bool density_ppe_fusable(const SceneConst& sc) {
    return (sc.flags & MPS_FLAG_SPP) != 0u && (sc.flags & MPS_FLAG_PRESSURE_EXPLICIT) == 0u;
}

void launch_density_set_ppe(const SceneConst& sc, const DeviceState& st, bool want_fp32, cudaStream_t s) {
    k_density_ppe<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, assembly_state(st, want_fp32));
    launch_ppe_layout(sc, st, want_fp32, s);
}

void launch_assign_pressure(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_assign_pressure<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_explicit_pressure(const SceneConst& sc, const DeviceState& st, int32_t* ok, cudaStream_t s) {
    k_explicit_pressure<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st, ok);
}

void launch_density_explicit_pressure(const SceneConst& sc, const DeviceState& st, int32_t* ok,
                                      cudaStream_t s) {
    k_density_explicit_pressure<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st, ok);
}

void launch_pressure_gradient(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    if (sc.flags & MPS_FLAG_GC)
        k_pressure_gradient_gc<0><<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
    else
        k_pressure_gradient<0><<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
    k_apply_du<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

// spp_sums: the fused density + assembly walk (k_density_ppe) ran on these positions with
// r_e^lap = r_e, so its SPP sums are the gradient's
void launch_pressure_gradient_cached(const SceneConst& sc, const DeviceState& st, bool spp_sums, cudaStream_t s) {
    const dim3 g(grid_for(sc.n, kWalkBlock));
    if (sc.flags & MPS_FLAG_GC) {
        if (spp_sums)
            k_pressure_gradient_gc<2><<<g, kWalkBlock, 0, s>>>(sc, st);
        else
            k_pressure_gradient_gc<1><<<g, kWalkBlock, 0, s>>>(sc, st);
    } else if (spp_sums) {
        k_pressure_gradient<2><<<g, kWalkBlock, 0, s>>>(sc, st);
    } else {
        k_pressure_gradient<1><<<g, kWalkBlock, 0, s>>>(sc, st);
    }
    k_apply_du<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

void launch_dynamic_stabilize(const SceneConst& sc, const DeviceState& st, cudaStream_t s) {
    k_dynamic_stabilize<<<grid_for(sc.n, kWalkBlock), kWalkBlock, 0, s>>>(sc, st);
    k_apply_du<<<grid_for(sc.n), kBlock, 0, s>>>(sc, st);
}

}  // namespace mpsgb
