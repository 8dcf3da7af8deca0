/*
 * mps_oracle.cpp - CPU oracle of the MPS time step.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++17 restatement of OpenMps's `Computer::ForwardTime` and the
 * classes it uses, written from the reference's behaviour:
 *   Environment  src/OpenMps/Environment.hpp:129-216
 *   Particle::W  src/OpenMps/Particle.hpp:71-75
 *   Grid         src/OpenMps/Grid.hpp:137-331 (cells), :334-559 (iterator order)
 *   Computer     src/OpenMps/Computer.hpp:565-1751
 * Boost uBLAS 2-vectors become two doubles; uBLAS `inner_prod` / `norm_2` on a
 * 2-vector are restated as `t = 0; t += a0*b0; t += a1*b1` (and sqrt of that),
 * which is how uBLAS evaluates them.  ViennaCL (used only for the CSR SpMV, dot
 * products and vector updates inside the hand-written CG, Computer.hpp:1382-1418)
 * becomes serial loops.  The expression order of every floating-point formula is
 * the reference's; build with -ffp-contract=off so no multiply-add is fused.
 *
 * The compile-time method switches of defines.hpp become runtime flags
 * (MPS_FLAG_*).  Two things are extensions, present on both sides of the parity
 * tests and absent from the reference:
 *   - a second (Laplacian) radius re_lap for viscosity and the PPE matrix, with
 *     its own n0/lambda; with re_lap == re everything reduces to the reference;
 *   - the CG stopping rule |b - A x| <= eps |b| (MPS_CRIT_RHS).
 *
 * Built twice from this file: serial (the parity oracle) and with OpenMP (the
 * timed CPU baseline; its dot products then reduce in thread order, as the
 * reference's ViennaCL-OpenMP backend does).  Nothing in the product links it.
 */
#include "mps_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#define ORACLE_PARALLEL_FOR _Pragma("omp parallel for schedule(static)")
#else
#define ORACLE_PARALLEL_FOR
#endif

namespace {

struct OracleError {
    int code;
    std::string msg;
};

/* Particle::W (Particle.hpp:71-75) */
inline double weight(double r, double re) { return ((0 < r) && (r < re)) ? (re / r - 1) : 0; }

/* uBLAS inner_prod of two 2-vectors */
inline double dot2(double a0, double a1, double b0, double b1) {
    double t = 0.0;
    t += a0 * b0;
    t += a1 * b1;
    return t;
}

/* n0 and lambda of a square lattice (Environment.hpp:163-215) */
void lattice_constants(double re_by_l0, double l0, double& n0, double& lambda) {
    const double re = re_by_l0 * l0;
    const int range = static_cast<int>(std::ceil(re_by_l0));
    n0 = 0;
    lambda = 0;
    for (int i = -range; i < range; i++) {
        for (int j = -range; j < range; j++) {
            if (!((i == 0) && (j == 0))) {
                const double x0 = i * l0;
                const double x1 = j * l0;
                const double r = std::sqrt(dot2(x0, x1, x0, x1));
                if (r < re) {
                    const double w = weight(r, re);
                    n0 += w;
                    lambda += r * r * w;
                }
            }
        }
    }
    lambda /= n0;
}

inline bool has(uint32_t flags, uint32_t f) { return (flags & f) != 0; }

/* Detail::InvertMatrix<2> (Computer.hpp:323-347): the inverse of [[a, b], [c, d]], or
 * val times the identity when the determinant is exactly zero.  out = {m00, m01, m10, m11}. */
void gc_invert(double a, double b, double c, double d, double val, double* out) {
    const double det = a * d - b * c;
    if (det == 0) {
        out[0] = val;
        out[1] = 0;
        out[2] = 0;
        out[3] = val;
        return;
    }
    out[0] = d / det;
    out[1] = -b / det;
    out[2] = -c / det;
    out[3] = a / det;
}

class Oracle {
public:
    mps_params prm;
    /* Environment */
    double t = 0, dt = 0;
    double n0 = 0, lambda = 0, n0_lap = 0, lambda_lap = 0;
    double max_dt = 0, max_dx = 0, l0 = 0, re = 0, re_lap = 0, nl = 0;
    /* Grid */
    int64_t gnx = 0, gnz = 0, max_per_cell = 0;
    std::vector<int64_t> cell_count;
    std::vector<int32_t> cell_slot;
    /* particles (Computer::particles, SoA) */
    std::vector<int32_t> type;
    std::vector<double> x, z, u, w, p, nd;
    std::vector<double> wall_x, wall_z;
    std::vector<double> n_wo_spp, ecs, ox, oz, dux, duz;
    /* neighbour lists: padded rows like Computer::neighbor (Computer.hpp:1763-1765) */
    int64_t nb_stride = 0;
    std::vector<int32_t> nb_count, nb;
    /* PPE (Computer::Ppe, Computer.hpp:480-537) */
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> col;
    std::vector<double> val, b, xs;
    int32_t criterion = MPS_CRIT_INITIAL_RESIDUAL;
    double eps = 1e-10;
    int32_t max_iters = 0;
    int32_t last_iters = 0;
    double last_rr0 = 0, last_rr = 0;
    std::string err;

    explicit Oracle(const mps_params& prm_) : prm(prm_) {
        const double re_by = prm.re_by_l0;
        const double rl_by = prm.re_lap_by_l0 > 0 ? prm.re_lap_by_l0 : prm.re_by_l0;
        l0 = prm.l0;
        re = re_by * l0;                                               /* Environment.hpp:145 */
        re_lap = rl_by * l0;
        if (has(prm.flags, MPS_FLAG_PRESSURE_EXPLICIT))
            max_dt = std::min(prm.max_dt, (prm.courant * l0) / prm.sound_speed); /* :135 */
        else
            max_dt = std::min(prm.max_dt, std::sqrt(2 * (prm.courant * l0) / prm.g)); /* :138 */
        max_dx = prm.courant * l0;                                     /* :143 */
        nl = std::max(re_by, rl_by) * l0 * (1 + prm.courant * 2);      /* :161 */
        lattice_constants(re_by, l0, n0, lambda);
        lattice_constants(rl_by, l0, n0_lap, lambda_lap);
        /* Grid.hpp:137-150 */
        gnx = static_cast<int64_t>(std::ceil((prm.max_x - prm.min_x) / nl)) + 2;
        gnz = static_cast<int64_t>(std::ceil((prm.max_z - prm.min_z) / nl)) + 2;
        const int64_t c = static_cast<int64_t>(std::ceil(nl / l0));
        max_per_cell = (c + 1) * (c + 1);
        cell_count.assign(static_cast<size_t>(gnx * gnz), 0);
        cell_slot.assign(static_cast<size_t>(gnx * gnz * max_per_cell), -1);
        nb_stride = max_per_cell * 9;
        criterion = prm.criterion;
        eps = prm.eps;
        max_iters = prm.max_cg_iters;
    }

    size_t count() const { return type.size(); }
    bool spp() const { return has(prm.flags, MPS_FLAG_SPP); }
    bool is_surface(double n) const { return n / n0 < prm.surface_ratio; } /* Computer.hpp:586-589 */

    void resize_aux() {
        const size_t n = count();
        n_wo_spp.resize(n, 0.0);
        ecs.resize(n, 0.0);
        ox.resize(n, 0.0);
        oz.resize(n, 0.0);
        dux.resize(n, 0.0);
        duz.resize(n, 0.0);
        nb_count.assign(n, 0);
        nb.assign(n * static_cast<size_t>(nb_stride), -1);
    }

    /* Grid::Block (Grid.hpp:250-254); false if outside [0, cells) or not finite */
    static bool block(double xv, double origin, double len, int64_t cells, int64_t& out) {
        const double f = std::floor((xv - origin) / len);
        if (!(f >= 0.0 && f < static_cast<double>(cells))) return false;
        out = static_cast<int64_t>(f);
        return true;
    }

    /* SearchNeighbor (Computer.hpp:698-756) with Grid::Store (Grid.hpp:276-331) */
    void search_neighbor() {
        std::fill(cell_count.begin(), cell_count.end(), 0);
        const size_t n = count();
        for (size_t i = 0; i < n; i++) {
            if (type[i] == MPS_TYPE_DISABLED) continue;
            int64_t bx, bz;
            const bool ok = block(x[i], prm.min_x, nl, gnx, bx) && block(z[i], prm.min_z, nl, gnz, bz);
            if (!ok) {
                type[i] = MPS_TYPE_DISABLED;
                continue;
            }
            const int64_t cell = bx * gnz + bz;
            const int64_t l = cell_count[cell]++;
            if (l >= max_per_cell) throw OracleError{MPS_ERR_CELL_OVERFLOW, "Too many particle in a block"};
            cell_slot[cell * max_per_cell + l] = static_cast<int32_t>(i);
        }
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_DISABLED) {
                nb_count[i] = 0;
                continue;
            }
            int64_t bx = 0, bz = 0;
            block(x[i], prm.min_x, nl, gnx, bx);
            block(z[i], prm.min_z, nl, gnz, bz);
            int32_t idx = 0;
            int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            /* the nine cells in Grid::Iterator order (Grid.hpp:393-401); out-of-range cells skipped */
            for (int64_t di = -1; di <= 1; di++) {
                for (int64_t dk = -1; dk <= 1; dk++) {
                    const int64_t cx = bx + di, cz = bz + dk;
                    if (cx < 0 || cx >= gnx || cz < 0 || cz >= gnz) continue;
                    const int64_t cell = cx * gnz + cz;
                    const int64_t cnt = cell_count[cell];
                    for (int64_t l = 0; l < cnt; l++) {
                        const int32_t j = cell_slot[cell * max_per_cell + l];
                        if ((static_cast<size_t>(j) != i) && (type[j] != MPS_TYPE_DISABLED)) {
                            const double ddx = x[i] - x[j];
                            const double ddz = z[i] - z[j];
                            const double r = std::sqrt(dot2(ddx, ddz, ddx, ddz)); /* Computer::R :568-572 */
                            if (r < nl) row[idx++] = j;
                        }
                    }
                }
            }
            nb_count[i] = idx;
        }
    }

    /*
     * The space-potential particle appended by AccumulateNeighbor with MPS_SPP
     * (Computer.hpp:664-692).  gx/gz hold sum W(r)*dx over the neighbours in
     * radius `radius`; returns true with its position when it contributes.
     */
    bool spp_particle(size_t i, double radius, double gx, double gz, double& xs_, double& zs_) const {
        const double thisN = n_wo_spp[i];
        gx /= n0;
        gz /= n0;
        if (thisN < n0) {
            const double r_g = std::sqrt(dot2(gx, gz, gx, gz));
            if (r_g > std::numeric_limits<double>::epsilon()) {
                const double w_spp = n0 - thisN;
                const double r_spp = radius / (w_spp + 1);
                const double s = r_spp / r_g;
                xs_ = x[i] - s * gx;
                zs_ = z[i] - s * gz;
                return true;
            }
        }
        return false;
    }

    /* ComputeNeighborDensities (Computer.hpp:780-833) */
    void density() {
        const size_t n = count();
        const double re2 = re * re;
        const bool use_spp = spp();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (use_spp) n_wo_spp[i] = n0;
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            double thisN = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) thisN += weight(std::sqrt(r2), re);
            }
            /* with SPP the virtual particle adds nothing here: nWithoutSpp[i] == n0 during the sum */
            if (use_spp) {
                n_wo_spp[i] = thisN;
                nd[i] = (thisN < n0) ? n0 : thisN; /* std::max(thisN, n0) */
            } else {
                nd[i] = thisN;
            }
        }
    }

    /* NeighborDensityVariationSpeed (Computer.hpp:838-872) */
    double density_variation(size_t i) const {
        if (has(prm.flags, MPS_FLAG_HS)) {
            if (spp() && n_wo_spp[i] < n0) return 0.0;
            const double re2 = re * re;
            double sum = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) {
                    const double du = u[j] - u[i];
                    const double dw = w[j] - w[i];
                    const double r = std::sqrt(dot2(dx, dz, dx, dz));
                    sum += dot2(dx, dz, du, dw) / (r * r * r);
                }
            }
            return -re * sum;
        }
        return (nd[i] - n0) / dt;
    }

    /* ComputeErrorCorrection (Computer.hpp:877-910) */
    void error_correction() {
        const size_t n = count();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            const double speed = density_variation(i);
            const double error = (nd[i] - n0) / n0;
            ecs[i] = std::abs(error) * speed + std::abs(speed) * error;
        }
    }

    /* Laplacian coefficient of the viscosity term (Computer.hpp:963-970) */
    double viscosity_coefficient(double r) const {
        if (has(prm.flags, MPS_FLAG_HL)) return prm.nu * 3.0 * re_lap / n0_lap / (r * r * r);
        const double wgt = weight(r, re_lap);
        return prm.nu * 2 * 2.0 / lambda_lap / n0_lap * wgt;
    }

    /* Laplacian coefficient of the PPE matrix (Computer.hpp:1290-1297) */
    double ppe_coefficient(double r) const {
        if (has(prm.flags, MPS_FLAG_HL)) return 3.0 * re_lap / n0_lap / (r * r * r);
        const double wgt = weight(r, re_lap);
        return (4.0 / lambda_lap / n0_lap) * wgt;
    }

    /* ComputeExplicitForces (Computer.hpp:914-1021) with static wall targets */
    void explicit_forces() {
        const size_t n = count();
        const double rl2 = re_lap * re_lap;
        const bool use_spp = spp();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double vx = 0.0, vz = 0.0, gx = 0.0, gz = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < rl2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double c = viscosity_coefficient(std::sqrt(r2));
                        vx += c * (u[j] - u[i]);
                        vz += c * (w[j] - w[i]);
                    } else {
                        vx += 0.0;
                        vz += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight(std::sqrt(r2), re_lap);
                        gx += wg * dx;
                        gz += wg * dz;
                    }
                }
            }
            double sxp, szp;
            if (use_spp && spp_particle(i, re_lap, gx, gz, sxp, szp)) {
                /* the virtual particle moves with u_i: its term is coefficient * (0, 0) */
                const double ddx = x[i] - sxp, ddz = z[i] - szp;
                const double c = viscosity_coefficient(std::sqrt(dot2(ddx, ddz, ddx, ddz)));
                vx += c * (u[i] - u[i]);
                vz += c * (w[i] - w[i]);
            }
            if (has(prm.flags, MPS_FLAG_CENTRAL_GRAVITY)) {
                /* CENTRAL_GRAVITY (Computer.hpp:925-932, :981-988): a += G_z c, c = x / |x| */
                const double g = -prm.g;
                const double r = std::sqrt(dot2(x[i], z[i], x[i], z[i]));
                const double cx = (r < l0 * 0.01) ? 0.0 : x[i] / r;
                const double cz = (r < l0 * 0.01) ? 0.0 : z[i] / r;
                dux[i] = vx + g * cx;
                duz[i] = vz + g * cz;
            } else {
                dux[i] = vx + 0.0; /* a = vis; a += G, G = (0, -g) (Environment.hpp:149) */
                duz[i] = vz + (-prm.g);
            }
        }
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_FLUID) {
                u[i] += dux[i] * dt;
                w[i] += duz[i] * dt;
                x[i] += u[i] * dt;
                z[i] += w[i] * dt;
            } else {
                /* positionWall(i, t, dt); u = (x_new - x_old) / dt (Computer.hpp:1015-1018) */
                const double nx_ = wall_x[i], nz_ = wall_z[i];
                u[i] = (nx_ - x[i]) / dt;
                w[i] = (nz_ - z[i]) / dt;
                x[i] = nx_;
                z[i] = nz_;
            }
        }
    }

    /* SaveX (Computer.hpp:1025-1039) */
    void save_x() {
        const size_t n = count();
        for (size_t i = 0; i < n; i++) {
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            ox[i] = x[i];
            oz[i] = z[i];
        }
    }

    bool ppe_alive(size_t i) const {
        if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) return false;
        if (!spp() && is_surface(nd[i])) return false;
        return true;
    }

    /* SetPressurePoissonEquation (Computer.hpp:1145-1356) */
    void set_ppe() {
        const size_t n = count();
        b.assign(n, 0.0);
        xs.assign(n, 0.0);
        const double rl2 = re_lap * re_lap;
        const bool use_spp = spp();
        const bool use_ecs = has(prm.flags, MPS_FLAG_ECS);
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (!ppe_alive(i)) {
                b[i] = 0;
                xs[i] = 0;
            } else {
                const double speed = density_variation(i);
                if (use_ecs) {
                    const double e = ecs[i];
                    b[i] = -prm.rho / (n0 * dt) * (speed + e);
                } else {
                    b[i] = -prm.rho / (n0 * dt) * speed;
                }
                xs[i] = p[i];
            }
        }
        std::vector<std::vector<std::pair<int32_t, double>>> rows(n);
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            auto& a_i = rows[i];
            if (!ppe_alive(i)) {
                a_i.emplace_back(static_cast<int32_t>(i), 1.0);
                continue;
            }
            double a_ii = 0.0, gx = 0.0, gz = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < rl2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double a_ij = ppe_coefficient(std::sqrt(r2));
                        if (use_spp || !is_surface(nd[j])) a_i.emplace_back(j, a_ij);
                        a_ii += -a_ij;
                    } else {
                        a_ii += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight(std::sqrt(r2), re_lap);
                        gx += wg * dx;
                        gz += wg * dz;
                    }
                }
            }
            double sxp, szp;
            if (use_spp && spp_particle(i, re_lap, gx, gz, sxp, szp)) {
                const double ddx = x[i] - sxp, ddz = z[i] - szp;
                const double a_s = ppe_coefficient(std::sqrt(dot2(ddx, ddz, ddx, ddz)));
                a_ii += -a_s; /* diagonal only: j = -1 is never stored (Computer.hpp:1299-1301) */
            }
            a_i.emplace_back(static_cast<int32_t>(i), a_ii);
        }
        /* uBLAS compressed_matrix keeps each row's columns ascending (Computer.hpp:1330-1350) */
        row_ptr.assign(n + 1, 0);
        for (size_t i = 0; i < n; i++) {
            std::sort(rows[i].begin(), rows[i].end(),
                      [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& c) {
                          return a.first < c.first;
                      });
            row_ptr[i + 1] = row_ptr[i] + static_cast<int64_t>(rows[i].size());
        }
        col.resize(static_cast<size_t>(row_ptr[n]));
        val.resize(static_cast<size_t>(row_ptr[n]));
        for (size_t i = 0; i < n; i++) {
            int64_t o = row_ptr[i];
            for (const auto& e : rows[i]) {
                col[static_cast<size_t>(o)] = e.first;
                val[static_cast<size_t>(o)] = e.second;
                o++;
            }
        }
    }

    void solve_ppe() {
        int32_t it = 0;
        double rr0 = 0, rr = 0;
        const int64_t n = static_cast<int64_t>(count());
        const int rc = cg_solve(n, row_ptr.data(), col.data(), val.data(), b.data(), xs.data(), eps,
                                criterion, max_iters, &it, &rr0, &rr);
        last_iters = it;
        last_rr0 = rr0;
        last_rr = rr;
        if (rc != MPS_OK)
            throw OracleError{rc, "Conjugate Gradient method couldn't solve Pressure Poison Equation"};
    }

    /* ComputeImplicitForces pressure assignment (Computer.hpp:1076-1097) */
    void assign_pressure() {
        const size_t n = count();
        const bool use_spp = spp();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            const double v = xs[i];
            p[i] = ((v < 0) || (!use_spp && is_surface(nd[i]))) ? 0 : v;
        }
    }

    /* ComputeImplicitForces with PRESSURE_EXPLICIT (Computer.hpp:1046-1067): every particle */
    void explicit_pressure() {
        const size_t n = count();
        const double c = prm.sound_speed;
        const double rho0 = prm.rho;
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            const double rho = rho0 / n0 * nd[i];
            p[i] = (rho <= rho0) ? 0 : c * c * (rho - rho0);
        }
    }

    /* ModifyByPressureGradient, MPS_GC branch (Computer.hpp:1457-1499, :1543-1563) */
    void pressure_gradient_gc() {
        const size_t n = count();
        const double re2 = re * re;
        const bool use_spp = spp();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            /* C^-1 = sum (W / r^2) dx dx^T over every neighbour within r_e, then the SPP
             * particle (a first AccumulateNeighbor, :1459-1470) */
            double m00 = 0.0, m01 = 0.0, m10 = 0.0, m11 = 0.0, gx = 0.0, gz = 0.0;
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) {
                    const double wg = weight(std::sqrt(r2), re);
                    const double t = wg / r2;
                    m00 += t * (dx * dx);
                    m01 += t * (dx * dz);
                    m10 += t * (dz * dx);
                    m11 += t * (dz * dz);
                    if (use_spp) {
                        gx += wg * dx;
                        gz += wg * dz;
                    }
                }
            }
            double sxp = 0.0, szp = 0.0;
            const bool has_spp = use_spp && spp_particle(i, re, gx, gz, sxp, szp);
            if (has_spp) {
                const double dx = sxp - x[i];
                const double dz = szp - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                const double t = weight(std::sqrt(r2), re) / r2;
                m00 += t * (dx * dx);
                m01 += t * (dx * dz);
                m10 += t * (dz * dx);
                m11 += t * (dz * dz);
            }
            double C[4];
            gc_invert(m00, m01, m10, m11, 2.0 / n0, C); /* InvertMatrix(invC, DIM / n0) :1472 */
            /* sum over non-dummy neighbours of (p_ij / r^2 W) C dx, prod(C, dx) row by row
             * from 0 (:1475-1496) */
            double sx = 0.0, sz = 0.0;
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double c = (p[j] + p[i]) / r2 * weight(std::sqrt(r2), re);
                        const double cx = (0.0 + C[0] * dx) + C[1] * dz;
                        const double cz = (0.0 + C[2] * dx) + C[3] * dz;
                        sx += c * cx;
                        sz += c * cz;
                    } else {
                        sx += 0.0;
                        sz += 0.0;
                    }
                }
            }
            if (has_spp) {
                const double dx = sxp - x[i];
                const double dz = szp - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                const double c = (0.0 + p[i]) / r2 * weight(std::sqrt(r2), re);
                const double cx = (0.0 + C[0] * dx) + C[1] * dz;
                const double cz = (0.0 + C[2] * dx) + C[3] * dz;
                sx += c * cx;
                sz += c * cz;
            }
            const double factor = -dt * nd[i] / (prm.rho * n0);
            dux[i] = factor * sx;
            duz[i] = factor * sz;
        }
        apply_du();
    }

    /* u += du; x += du dt for fluid particles (Computer.hpp:1543-1563) */
    void apply_du() {
        const size_t n = count();
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            u[i] += dux[i];
            w[i] += duz[i];
            x[i] += dux[i] * dt;
            z[i] += duz[i] * dt;
        }
    }

    /* ModifyByPressureGradient, midpoint branch (Computer.hpp:1433-1521, :1543-1563) */
    void pressure_gradient() {
        if (has(prm.flags, MPS_FLAG_GC)) {
            pressure_gradient_gc();
            return;
        }
        const size_t n = count();
        const double re2 = re * re;
        const bool use_spp = spp();
        const double factor = -dt / prm.rho * 2.0 / n0;
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double sx = 0.0, sz = 0.0, gx = 0.0, gz = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) {
                    const double wg = weight(std::sqrt(r2), re);
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double c = (p[j] + p[i]) / r2 * wg;
                        sx += c * dx;
                        sz += c * dz;
                    } else {
                        sx += 0.0;
                        sz += 0.0;
                    }
                    if (use_spp) {
                        gx += wg * dx;
                        gz += wg * dz;
                    }
                }
            }
            double sxp, szp;
            if (use_spp && spp_particle(i, re, gx, gz, sxp, szp)) {
                /* virtual particle: p = 0, type fluid (Computer.hpp:682-689) */
                const double dx = sxp - x[i];
                const double dz = szp - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                const double c = (0.0 + p[i]) / r2 * weight(std::sqrt(r2), re);
                sx += c * dx;
                sz += c * dz;
            }
            dux[i] = factor * sx;
            duz[i] = factor * sz;
        }
        apply_du();
    }

    /* DynamicStabilize (Computer.hpp:1568-1656) */
    void dynamic_stabilize() {
        const size_t n = count();
        const double re2 = re * re;
        const double d = l0 - max_dx;
        const double d2 = d * d;
        const bool use_spp = spp();
        const double factor = -1.0 / (2 * dt * n0);
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double sx = 0.0, sz = 0.0, gx = 0.0, gz = 0.0;
            const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int32_t k = 0; k < nb_count[i]; k++) {
                const int32_t j = row[k];
                if (static_cast<size_t>(j) == i) continue;
                const double dx = x[j] - x[i];
                const double dz = z[j] - z[i];
                const double r2 = dot2(dx, dz, dx, dz);
                if (r2 < re2) {
                    if (type[j] != MPS_TYPE_DUMMY && r2 < d2) {
                        const double dx0 = ox[j] - ox[i];
                        const double dz0 = oz[j] - oz[i];
                        const double nrm = std::sqrt(dot2(dx0, dz0, dx0, dz0));
                        const double ex = dx0 / nrm;
                        const double ez = dz0 / nrm;
                        const double r_par = dot2(dx, dz, ex, ez);
                        const double px = dx - r_par * ex;
                        const double pz = dz - r_par * ez;
                        const double r_perp2 = dot2(px, pz, px, pz);
                        const double m = std::sqrt(d2 - r_perp2) - r_par;
                        sx += m * ex;
                        sz += m * ez;
                    } else {
                        sx += 0.0;
                        sz += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight(std::sqrt(r2), re);
                        gx += wg * dx;
                        gz += wg * dz;
                    }
                }
            }
            double sxp, szp;
            if (use_spp && spp_particle(i, re, gx, gz, sxp, szp)) {
                sx += 0.0; /* the virtual particle (j < 0) is excluded (Computer.hpp:1597-1598) */
                sz += 0.0;
            }
            dux[i] = factor * sx;
            duz[i] = factor * sz;
        }
        ORACLE_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            u[i] += dux[i];
            w[i] += duz[i];
            x[i] += dux[i] * dt;
            z[i] += duz[i] * dt;
        }
    }

    /* DetermineDt (Computer.hpp:759-777) */
    double determine_dt() const {
        const size_t n = count();
        if (n == 0) return max_dt;
        size_t best = 0;
        for (size_t i = 1; i < n; i++) {
            if (dot2(u[best], w[best], u[best], w[best]) < dot2(u[i], w[i], u[i], w[i])) best = i;
        }
        const double maxU = std::sqrt(dot2(u[best], w[best], u[best], w[best]));
        if (maxU == 0) return max_dt;
        const double a = max_dx / maxU;
        return (max_dt < a) ? max_dt : a; /* std::min(a, MaxDt) */
    }

    void begin_step(double dt_) {
        dt = dt_; /* Computer.hpp:1703-1706 */
        t += dt;
    }

    /* ForwardTime(dt) (Computer.hpp:1700-1742) */
    void forward_time(double dt_) {
        if (!(dt_ > 0)) dt_ = determine_dt();
        begin_step(dt_);
        search_neighbor();
        density();
        if (has(prm.flags, MPS_FLAG_ECS)) error_correction();
        explicit_forces();
        density();
        if (has(prm.flags, MPS_FLAG_DS)) save_x();
        if (has(prm.flags, MPS_FLAG_PRESSURE_EXPLICIT)) {
            explicit_pressure();
        } else {
            set_ppe();
            solve_ppe();
            assign_pressure();
        }
        pressure_gradient();
        if (has(prm.flags, MPS_FLAG_DS)) dynamic_stabilize();
    }

    /*
     * SolvePressurePoissonEquation (Computer.hpp:1359-1429) on CSR (A, b, x).
     * ViennaCL's prod / inner_prod / vector updates are restated as loops.
     */
    static int cg_solve(int64_t n, const int64_t* rp, const int32_t* cl, const double* va,
                        const double* bb, double* xx, double eps_, int32_t crit, int32_t maxit,
                        int32_t* iters, double* rr0_out, double* rr_out) {
        std::vector<double> r(static_cast<size_t>(n)), pp(static_cast<size_t>(n)),
            Ap(static_cast<size_t>(n));
        auto spmv = [&](const double* v, double* out) {
            ORACLE_PARALLEL_FOR
            for (int64_t i = 0; i < n; i++) {
                double s = 0.0;
                for (int64_t k = rp[i]; k < rp[i + 1]; k++) s += va[k] * v[cl[k]];
                out[i] = s;
            }
        };
        auto dot = [&](const double* a, const double* c) {
            double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) schedule(static)
#endif
            for (int64_t i = 0; i < n; i++) s += a[i] * c[i];
            return s;
        };
        spmv(xx, Ap.data());
        ORACLE_PARALLEL_FOR
        for (int64_t i = 0; i < n; i++) {
            r[i] = bb[i] - Ap[i];
            pp[i] = r[i];
        }
        double rr = dot(r.data(), r.data());
        double threshold = rr * eps_ * eps_;
        if (crit == MPS_CRIT_RHS) {
            const double bnorm2 = dot(bb, bb);
            if (bnorm2 > 0) threshold = bnorm2 * eps_ * eps_;
        }
        if (rr0_out) *rr0_out = rr;
        bool converged = (crit == MPS_CRIT_RHS) ? (rr < threshold || rr == 0) : (threshold == 0);
        const int64_t limit = (maxit > 0) ? maxit : n;
        int32_t it = 0;
        double rr_last = rr;
        for (int64_t k = 0; (k < limit) && (!converged); k++) {
            spmv(pp.data(), Ap.data());
            const double alpha = rr / dot(pp.data(), Ap.data());
            ORACLE_PARALLEL_FOR
            for (int64_t i = 0; i < n; i++) {
                xx[i] += alpha * pp[i];
                r[i] -= alpha * Ap[i];
            }
            const double rrNew = dot(r.data(), r.data());
            rr_last = rrNew;
            converged = (rrNew < threshold);
            if (!converged) {
                const double beta = rrNew / rr;
                ORACLE_PARALLEL_FOR
                for (int64_t i = 0; i < n; i++) pp[i] = r[i] + beta * pp[i];
                rr = rrNew;
            }
            it++;
        }
        if (iters) *iters = it;
        if (rr_out) *rr_out = rr_last;
        return converged ? MPS_OK : MPS_ERR_CG_NOT_CONVERGED;
    }
};

template <class F>
int guarded(oracle_handle* h, F f);

}  // namespace

struct oracle_handle {
    Oracle* o;
};

namespace {
template <class F>
int guarded(oracle_handle* h, F f) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    try {
        f(*h->o);
        h->o->err.clear();
        return MPS_OK;
    } catch (const OracleError& e) {
        h->o->err = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        h->o->err = e.what();
        return MPS_ERR_STATE;
    }
}

template <class T>
void copy_out(const std::vector<T>& v, T* dst) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}
template <class T>
void copy_in(std::vector<T>& v, const T* src) {
    if (src && !v.empty()) std::memcpy(v.data(), src, v.size() * sizeof(T));
}
}  // namespace

extern "C" {

int oracle_create(const mps_params* prm, oracle_handle** out) {
    if (!prm || !out) return MPS_ERR_INVALID_ARGUMENT;
    if (!(prm->l0 > 0) || !(prm->re_by_l0 > 0) || !(prm->g >= 0) || !(prm->max_x > prm->min_x) ||
        !(prm->max_z > prm->min_z))
        return MPS_ERR_INVALID_ARGUMENT;
    auto* h = new oracle_handle;
    h->o = new Oracle(*prm);
    *out = h;
    return MPS_OK;
}

void oracle_destroy(oracle_handle* h) {
    if (!h) return;
    delete h->o;
    delete h;
}

const char* oracle_last_error(const oracle_handle* h) { return (h && h->o) ? h->o->err.c_str() : ""; }

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_add_particles(oracle_handle* h, int64_t n, const int32_t* type, const double* x,
                         const double* z, const double* u, const double* w, const double* p,
                         const double* nd) {
    if (n < 0 || (n > 0 && (!type || !x || !z))) return MPS_ERR_INVALID_ARGUMENT;
    return guarded(h, [&](Oracle& o) {
        for (int64_t i = 0; i < n; i++) {
            o.type.push_back(type[i]);
            o.x.push_back(x[i]);
            o.z.push_back(z[i]);
            o.u.push_back(u ? u[i] : 0.0);
            o.w.push_back(w ? w[i] : 0.0);
            o.p.push_back(p ? p[i] : 0.0);
            o.nd.push_back(nd ? nd[i] : 0.0);
            o.wall_x.push_back(x[i]);
            o.wall_z.push_back(z[i]);
        }
        o.resize_aux();
    });
}

int64_t oracle_particle_count(const oracle_handle* h) {
    return (h && h->o) ? static_cast<int64_t>(h->o->count()) : -1;
}

int oracle_get_particles(const oracle_handle* h, int32_t* type, double* x, double* z, double* u,
                         double* w, double* p, double* nd) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    copy_out(o.type, type);
    copy_out(o.x, x);
    copy_out(o.z, z);
    copy_out(o.u, u);
    copy_out(o.w, w);
    copy_out(o.p, p);
    copy_out(o.nd, nd);
    return MPS_OK;
}

int oracle_set_particles(oracle_handle* h, const int32_t* type, const double* x, const double* z,
                         const double* u, const double* w, const double* p, const double* nd) {
    return guarded(h, [&](Oracle& o) {
        copy_in(o.type, type);
        copy_in(o.x, x);
        copy_in(o.z, z);
        copy_in(o.u, u);
        copy_in(o.w, w);
        copy_in(o.p, p);
        copy_in(o.nd, nd);
    });
}

int oracle_set_wall_positions(oracle_handle* h, const double* wx, const double* wz) {
    return guarded(h, [&](Oracle& o) {
        copy_in(o.wall_x, wx);
        copy_in(o.wall_z, wz);
    });
}

int oracle_set_solver(oracle_handle* h, int32_t criterion, double eps, int32_t max_iters) {
    return guarded(h, [&](Oracle& o) {
        o.criterion = criterion;
        o.eps = eps;
        o.max_iters = max_iters;
    });
}

int oracle_forward_time(oracle_handle* h, double dt) {
    return guarded(h, [&](Oracle& o) { o.forward_time(dt); });
}

int oracle_get_environment(const oracle_handle* h, mps_environment* env) {
    if (!h || !h->o || !env) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    std::memset(env, 0, sizeof(*env));
    env->t = o.t;
    env->dt = o.dt;
    env->n0 = o.n0;
    env->lambda = o.lambda;
    env->n0_lap = o.n0_lap;
    env->lambda_lap = o.lambda_lap;
    env->max_dt = o.max_dt;
    env->max_dx = o.max_dx;
    env->l0 = o.l0;
    env->re = o.re;
    env->re_lap = o.re_lap;
    env->neighbor_length = o.nl;
    env->rho = o.prm.rho;
    env->nu = o.prm.nu;
    env->g = o.prm.g;
    env->min_x = o.prm.min_x;
    env->min_z = o.prm.min_z;
    env->max_x = o.prm.max_x;
    env->max_z = o.prm.max_z;
    env->grid_nx = o.gnx;
    env->grid_nz = o.gnz;
    env->grid_max_per_cell = o.max_per_cell;
    return MPS_OK;
}

int oracle_get_stats(const oracle_handle* h, int32_t* cg_iterations, double* rr0, double* rr,
                     int64_t* ppe_nnz, int64_t* neighbor_total) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    if (cg_iterations) *cg_iterations = o.last_iters;
    if (rr0) *rr0 = o.last_rr0;
    if (rr) *rr = o.last_rr;
    if (ppe_nnz) *ppe_nnz = o.row_ptr.empty() ? 0 : o.row_ptr.back();
    if (neighbor_total) {
        int64_t s = 0;
        for (auto c : o.nb_count) s += c;
        *neighbor_total = s;
    }
    return MPS_OK;
}

int oracle_stage_begin_step(oracle_handle* h, double dt) {
    return guarded(h, [&](Oracle& o) { o.begin_step(dt); });
}
int oracle_stage_search_neighbor(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.search_neighbor(); });
}
int oracle_stage_density(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.density(); });
}
int oracle_stage_error_correction(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.error_correction(); });
}
int oracle_stage_explicit(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.explicit_forces(); });
}
int oracle_stage_save_x(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.save_x(); });
}
int oracle_stage_set_ppe(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.set_ppe(); });
}
int oracle_stage_solve_ppe(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.solve_ppe(); });
}
int oracle_stage_assign_pressure(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) {
        if (has(o.prm.flags, MPS_FLAG_PRESSURE_EXPLICIT))
            o.explicit_pressure();
        else
            o.assign_pressure();
    });
}
void oracle_gc_invert(const double* m, double val, double* out) { gc_invert(m[0], m[1], m[2], m[3], val, out); }
int oracle_stage_pressure_gradient(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.pressure_gradient(); });
}
int oracle_stage_dynamic_stabilize(oracle_handle* h) {
    return guarded(h, [&](Oracle& o) { o.dynamic_stabilize(); });
}
int oracle_stage_density_variation(oracle_handle* h, double* speed) {
    if (!speed) return MPS_ERR_INVALID_ARGUMENT;
    return guarded(h, [&](Oracle& o) {
        for (size_t i = 0; i < o.count(); i++) {
            const bool alive = o.type[i] != MPS_TYPE_DUMMY && o.type[i] != MPS_TYPE_DISABLED;
            speed[i] = alive ? o.density_variation(i) : 0.0;
        }
    });
}
double oracle_determine_dt(oracle_handle* h) { return (h && h->o) ? h->o->determine_dt() : 0.0; }

int oracle_get_neighbors(const oracle_handle* h, int32_t* counts, int32_t* list, int64_t capacity,
                         int64_t* total) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    int64_t off = 0;
    for (size_t i = 0; i < o.count(); i++) {
        const int32_t c = o.nb_count.empty() ? 0 : o.nb_count[i];
        if (counts) counts[i] = c;
        for (int32_t k = 0; k < c; k++) {
            if (list && off < capacity) list[off] = o.nb[i * static_cast<size_t>(o.nb_stride) + k];
            off++;
        }
    }
    if (total) *total = off;
    return (list && off > capacity) ? MPS_ERR_INVALID_ARGUMENT : MPS_OK;
}

int oracle_get_ppe(const oracle_handle* h, int64_t* row_ptr, int32_t* col, double* val, double* b,
                   double* x, int64_t capacity, int64_t* nnz) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    const int64_t total = o.row_ptr.empty() ? 0 : o.row_ptr.back();
    if (nnz) *nnz = total;
    copy_out(o.row_ptr, row_ptr);
    if ((col || val) && total > capacity) return MPS_ERR_INVALID_ARGUMENT;
    copy_out(o.col, col);
    copy_out(o.val, val);
    copy_out(o.b, b);
    copy_out(o.xs, x);
    return MPS_OK;
}

int oracle_set_ppe_x(oracle_handle* h, const double* x) {
    return guarded(h, [&](Oracle& o) { copy_in(o.xs, x); });
}

int oracle_get_aux(const oracle_handle* h, double* n_without_spp, double* ecs, double* ox,
                   double* oz) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle& o = *h->o;
    copy_out(o.n_wo_spp, n_without_spp);
    copy_out(o.ecs, ecs);
    copy_out(o.ox, ox);
    copy_out(o.oz, oz);
    return MPS_OK;
}

int oracle_set_aux(oracle_handle* h, const double* n_without_spp, const double* ecs,
                   const double* ox, const double* oz) {
    return guarded(h, [&](Oracle& o) {
        copy_in(o.n_wo_spp, n_without_spp);
        copy_in(o.ecs, ecs);
        copy_in(o.ox, ox);
        copy_in(o.oz, oz);
    });
}

int oracle_cg_solve_csr(int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val,
                        const double* b, double* x, double eps, int32_t criterion,
                        int32_t max_iters, int32_t* iterations, double* rr0, double* rr) {
    if (n < 0 || (n > 0 && (!row_ptr || !b || !x))) return MPS_ERR_INVALID_ARGUMENT;
    return Oracle::cg_solve(n, row_ptr, col, val, b, x, eps, criterion, max_iters, iterations, rr0,
                            rr);
}

}  // extern "C"
