/*
 * mps_oracle3.cpp - CPU oracle of the three-dimensional MPS time step.  TEST
 * INFRASTRUCTURE ONLY.
 *
 * The DIM3 build of OpenMps (defines.hpp:9-11) restated in plain C++17, from the
 * reference's behaviour with DIM = 3:
 *   Environment  src/OpenMps/Environment.hpp:129-216 (the x, y, z lattice loops)
 *   Grid         src/OpenMps/Grid.hpp:137-331 (cells [x][y][z]), :364-391 (the 27 cells)
 *   Computer     src/OpenMps/Computer.hpp:565-1751 with 3-vectors; uBLAS inner_prod /
 *                norm_2 / prod on 3-vectors as t = 0; t += a0 b0; t += a1 b1; t += a2 b2
 *   GC           Detail::InvertMatrix<3> (Computer.hpp:364-422)
 * The row capacity of a neighbour list is the reference's MaxNeighborCount, 9
 * maxPerCell (Computer.hpp:1136-1140); a longer row is reported as an error instead of
 * written past its end.  The PPE solve is the reference CG of mps_oracle.cpp.  Build
 * with -ffp-contract=off.  Nothing in the product links it.
 */
#include "mps_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#define ORACLE3_PARALLEL_FOR _Pragma("omp parallel for schedule(static)")
#else
#define ORACLE3_PARALLEL_FOR
#endif

namespace {

struct Oracle3Error {
    int code;
    std::string msg;
};

/* Particle::W (Particle.hpp:71-75) */
inline double weight3(double r, double re) { return ((0 < r) && (r < re)) ? (re / r - 1) : 0; }

/* uBLAS inner_prod of two 3-vectors */
inline double dot3(double a0, double a1, double a2, double b0, double b1, double b2) {
    double t = 0.0;
    t += a0 * b0;
    t += a1 * b1;
    t += a2 * b2;
    return t;
}

inline bool flag(uint32_t flags, uint32_t f) { return (flags & f) != 0; }

/* Environment.hpp:166-215, DIM3: i (x) outer, then j (y), then k (z) */
void lattice_constants3(double re_by_l0, double l0, double& n0, double& lambda) {
    const double re = re_by_l0 * l0;
    const int range = static_cast<int>(std::ceil(re_by_l0));
    n0 = 0;
    lambda = 0;
    for (int i = -range; i < range; i++)
        for (int j = -range; j < range; j++)
            for (int k = -range; k < range; k++) {
                if ((i == 0) && (j == 0) && (k == 0)) continue;
                const double x0 = i * l0, x1 = j * l0, x2 = k * l0;
                const double r = std::sqrt(dot3(x0, x1, x2, x0, x1, x2));
                if (r < re) {
                    const double w = weight3(r, re);
                    n0 += w;
                    lambda += r * r * w;
                }
            }
    lambda /= n0;
}

class Oracle3 {
public:
    mps_params prm;
    double t = 0, dt = 0;
    double n0 = 0, lambda = 0, n0_lap = 0, lambda_lap = 0;
    double max_dt = 0, max_dx = 0, l0 = 0, re = 0, re_lap = 0, nl = 0;
    int64_t gnx = 0, gny = 0, gnz = 0, max_per_cell = 0;
    std::vector<int64_t> cell_count;
    std::vector<int32_t> cell_slot;
    std::vector<int32_t> type;
    std::vector<double> x, y, z, u, v, w, p, nd;
    std::vector<double> wall_x, wall_y, wall_z;
    std::vector<double> n_wo_spp, ecs, ox, oy, oz, dux, duy, duz;
    int64_t nb_stride = 0;
    std::vector<int32_t> nb_count, nb;
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> col;
    std::vector<double> val, b, xs;
    int32_t last_iters = 0;
    double last_rr0 = 0, last_rr = 0;
    std::string err;

    explicit Oracle3(const mps_params& prm_) : prm(prm_) {
        const double re_by = prm.re_by_l0;
        const double rl_by = prm.re_lap_by_l0 > 0 ? prm.re_lap_by_l0 : prm.re_by_l0;
        l0 = prm.l0;
        re = re_by * l0;
        re_lap = rl_by * l0;
        if (flag(prm.flags, MPS_FLAG_PRESSURE_EXPLICIT))
            max_dt = std::min(prm.max_dt, (prm.courant * l0) / prm.sound_speed); /* :135 */
        else
            max_dt = std::min(prm.max_dt, std::sqrt(2 * (prm.courant * l0) / prm.g)); /* :138 */
        max_dx = prm.courant * l0;
        nl = std::max(re_by, rl_by) * l0 * (1 + prm.courant * 2);
        lattice_constants3(re_by, l0, n0, lambda);
        lattice_constants3(rl_by, l0, n0_lap, lambda_lap);
        gnx = static_cast<int64_t>(std::ceil((prm.max_x - prm.min_x) / nl)) + 2;
        gny = static_cast<int64_t>(std::ceil((prm.max_y - prm.min_y) / nl)) + 2;
        gnz = static_cast<int64_t>(std::ceil((prm.max_z - prm.min_z) / nl)) + 2;
        const int64_t c = static_cast<int64_t>(std::ceil(nl / l0));
        max_per_cell = (c + 1) * (c + 1) * (c + 1);
        cell_count.assign(static_cast<size_t>(gnx * gny * gnz), 0);
        cell_slot.assign(static_cast<size_t>(gnx * gny * gnz * max_per_cell), -1);
        nb_stride = max_per_cell * 9;
    }

    size_t count() const { return type.size(); }
    bool spp() const { return flag(prm.flags, MPS_FLAG_SPP); }
    bool is_surface(double n) const { return n / n0 < prm.surface_ratio; }

    void resize_aux() {
        const size_t n = count();
        for (auto* a : {&n_wo_spp, &ecs, &ox, &oy, &oz, &dux, &duy, &duz}) a->resize(n, 0.0);
        nb_count.assign(n, 0);
        nb.assign(n * static_cast<size_t>(nb_stride), -1);
    }

    static bool block(double xv, double origin, double len, int64_t cells, int64_t& out) {
        const double f = std::floor((xv - origin) / len);
        if (!(f >= 0.0 && f < static_cast<double>(cells))) return false;
        out = static_cast<int64_t>(f);
        return true;
    }
    int64_t cell_of(int64_t bx, int64_t by, int64_t bz) const { return (bx * gny + by) * gnz + bz; }

    /* SearchNeighbor (Computer.hpp:698-756) with Grid::Store and the 27-cell iterator */
    void search_neighbor() {
        std::fill(cell_count.begin(), cell_count.end(), 0);
        const size_t n = count();
        for (size_t i = 0; i < n; i++) {
            if (type[i] == MPS_TYPE_DISABLED) continue;
            int64_t bx, by, bz;
            const bool ok = block(x[i], prm.min_x, nl, gnx, bx) && block(y[i], prm.min_y, nl, gny, by) &&
                            block(z[i], prm.min_z, nl, gnz, bz);
            if (!ok) {
                type[i] = MPS_TYPE_DISABLED;
                continue;
            }
            const int64_t cell = cell_of(bx, by, bz);
            const int64_t l = cell_count[cell]++;
            if (l >= max_per_cell) throw Oracle3Error{MPS_ERR_CELL_OVERFLOW, "Too many particle in a block"};
            cell_slot[cell * max_per_cell + l] = static_cast<int32_t>(i);
        }
        std::vector<char> overflow(n, 0);
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_DISABLED) {
                nb_count[i] = 0;
                continue;
            }
            int64_t bx = 0, by = 0, bz = 0;
            block(x[i], prm.min_x, nl, gnx, bx);
            block(y[i], prm.min_y, nl, gny, by);
            block(z[i], prm.min_z, nl, gnz, bz);
            int64_t idx = 0;
            int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
            for (int64_t di = -1; di <= 1; di++)
                for (int64_t dj = -1; dj <= 1; dj++)
                    for (int64_t dk = -1; dk <= 1; dk++) {
                        const int64_t cx = bx + di, cy = by + dj, cz = bz + dk;
                        if (cx < 0 || cx >= gnx || cy < 0 || cy >= gny || cz < 0 || cz >= gnz) continue;
                        const int64_t cell = cell_of(cx, cy, cz);
                        for (int64_t l = 0; l < cell_count[cell]; l++) {
                            const int32_t j = cell_slot[cell * max_per_cell + l];
                            if ((static_cast<size_t>(j) == i) || (type[j] == MPS_TYPE_DISABLED)) continue;
                            const double ddx = x[i] - x[j], ddy = y[i] - y[j], ddz = z[i] - z[j];
                            const double r = std::sqrt(dot3(ddx, ddy, ddz, ddx, ddy, ddz));
                            if (r < nl) {
                                if (idx < nb_stride)
                                    row[idx] = j;
                                else
                                    overflow[i] = 1;
                                idx++;
                            }
                        }
                    }
            nb_count[i] = static_cast<int32_t>(std::min(idx, nb_stride));
        }
        if (std::find(overflow.begin(), overflow.end(), 1) != overflow.end())
            throw Oracle3Error{MPS_ERR_DEVICE_CHECK, "neighbour row longer than 9 maxPerCell"};
    }

    /* the SPP particle of AccumulateNeighbor (Computer.hpp:664-692) */
    bool spp_particle(size_t i, double radius, double gx, double gy, double gz, double& xs_, double& ys_,
                      double& zs_) const {
        const double thisN = n_wo_spp[i];
        gx /= n0;
        gy /= n0;
        gz /= n0;
        if (thisN < n0) {
            const double r_g = std::sqrt(dot3(gx, gy, gz, gx, gy, gz));
            if (r_g > std::numeric_limits<double>::epsilon()) {
                const double w_spp = n0 - thisN;
                const double r_spp = radius / (w_spp + 1);
                const double s = r_spp / r_g;
                xs_ = x[i] - s * gx;
                ys_ = y[i] - s * gy;
                zs_ = z[i] - s * gz;
                return true;
            }
        }
        return false;
    }

    template <class F>
    void for_neighbors(size_t i, F f) const {
        const int32_t* row = &nb[i * static_cast<size_t>(nb_stride)];
        for (int32_t k = 0; k < nb_count[i]; k++) {
            const int32_t j = row[k];
            if (static_cast<size_t>(j) == i) continue;
            f(static_cast<size_t>(j), x[j] - x[i], y[j] - y[i], z[j] - z[i]);
        }
    }

    /* ComputeNeighborDensities (Computer.hpp:780-833) */
    void density() {
        const size_t n = count();
        const double re2 = re * re;
        const bool use_spp = spp();
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (use_spp) n_wo_spp[i] = n0;
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            double thisN = 0.0;
            for_neighbors(i, [&](size_t, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < re2) thisN += weight3(std::sqrt(r2), re);
            });
            if (use_spp) {
                n_wo_spp[i] = thisN;
                nd[i] = (thisN < n0) ? n0 : thisN;
            } else {
                nd[i] = thisN;
            }
        }
    }

    /* NeighborDensityVariationSpeed (Computer.hpp:838-872) */
    double density_variation(size_t i) const {
        if (flag(prm.flags, MPS_FLAG_HS)) {
            if (spp() && n_wo_spp[i] < n0) return 0.0;
            const double re2 = re * re;
            double sum = 0.0;
            for_neighbors(i, [&](size_t j, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < re2) {
                    const double r = std::sqrt(r2);
                    sum += dot3(dx, dy, dz, u[j] - u[i], v[j] - v[i], w[j] - w[i]) / (r * r * r);
                }
            });
            return -re * sum;
        }
        return (nd[i] - n0) / dt;
    }

    /* ComputeErrorCorrection (Computer.hpp:877-910) */
    void error_correction() {
        const size_t n = count();
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            const double speed = density_variation(i);
            const double error = (nd[i] - n0) / n0;
            ecs[i] = std::abs(error) * speed + std::abs(speed) * error;
        }
    }

    /* Computer.hpp:963-970 and :1290-1297 with DIM = 3 */
    double viscosity_coefficient(double r) const {
        if (flag(prm.flags, MPS_FLAG_HL)) return prm.nu * 2.0 * re_lap / n0_lap / (r * r * r);
        return prm.nu * 2 * 3.0 / lambda_lap / n0_lap * weight3(r, re_lap);
    }
    double ppe_coefficient(double r) const {
        if (flag(prm.flags, MPS_FLAG_HL)) return 2.0 * re_lap / n0_lap / (r * r * r);
        return (6.0 / lambda_lap / n0_lap) * weight3(r, re_lap);
    }

    /* ComputeExplicitForces (Computer.hpp:914-1021), G = (0, 0, -g), static wall targets */
    void explicit_forces() {
        const size_t n = count();
        const double rl2 = re_lap * re_lap;
        const bool use_spp = spp();
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double ax = 0.0, ay = 0.0, az = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
            for_neighbors(i, [&](size_t j, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < rl2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double c = viscosity_coefficient(std::sqrt(r2));
                        ax += c * (u[j] - u[i]);
                        ay += c * (v[j] - v[i]);
                        az += c * (w[j] - w[i]);
                    } else {
                        ax += 0.0;
                        ay += 0.0;
                        az += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight3(std::sqrt(r2), re_lap);
                        gx += wg * dx;
                        gy += wg * dy;
                        gz += wg * dz;
                    }
                }
            });
            double sxp, syp, szp;
            if (use_spp && spp_particle(i, re_lap, gx, gy, gz, sxp, syp, szp)) {
                const double ddx = x[i] - sxp, ddy = y[i] - syp, ddz = z[i] - szp;
                const double c = viscosity_coefficient(std::sqrt(dot3(ddx, ddy, ddz, ddx, ddy, ddz)));
                ax += c * (u[i] - u[i]);
                ay += c * (v[i] - v[i]);
                az += c * (w[i] - w[i]);
            }
            if (flag(prm.flags, MPS_FLAG_CENTRAL_GRAVITY)) { /* Computer.hpp:925-932, :981-988 */
                const double g = -prm.g;
                const double r = std::sqrt(dot3(x[i], y[i], z[i], x[i], y[i], z[i]));
                const bool zero = r < l0 * 0.01;
                dux[i] = ax + g * (zero ? 0.0 : x[i] / r);
                duy[i] = ay + g * (zero ? 0.0 : y[i] / r);
                duz[i] = az + g * (zero ? 0.0 : z[i] / r);
            } else {
                dux[i] = ax + 0.0;
                duy[i] = ay + 0.0;
                duz[i] = az + (-prm.g);
            }
        }
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] == MPS_TYPE_FLUID) {
                u[i] += dux[i] * dt;
                v[i] += duy[i] * dt;
                w[i] += duz[i] * dt;
                x[i] += u[i] * dt;
                y[i] += v[i] * dt;
                z[i] += w[i] * dt;
            } else {
                const double nx = wall_x[i], ny = wall_y[i], nz = wall_z[i];
                u[i] = (nx - x[i]) / dt;
                v[i] = (ny - y[i]) / dt;
                w[i] = (nz - z[i]) / dt;
                x[i] = nx;
                y[i] = ny;
                z[i] = nz;
            }
        }
    }

    /* SaveX (Computer.hpp:1025-1039) */
    void save_x() {
        for (size_t i = 0; i < count(); i++) {
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            ox[i] = x[i];
            oy[i] = y[i];
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
        const bool use_ecs = flag(prm.flags, MPS_FLAG_ECS);
        std::vector<std::vector<std::pair<int32_t, double>>> rows(n);
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            auto& a_i = rows[i];
            if (!ppe_alive(i)) {
                a_i.emplace_back(static_cast<int32_t>(i), 1.0);
                continue;
            }
            const double speed = density_variation(i);
            b[i] = use_ecs ? -prm.rho / (n0 * dt) * (speed + ecs[i]) : -prm.rho / (n0 * dt) * speed;
            xs[i] = p[i];
            double a_ii = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
            for_neighbors(i, [&](size_t j, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < rl2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        const double a_ij = ppe_coefficient(std::sqrt(r2));
                        if (use_spp || !is_surface(nd[j])) a_i.emplace_back(static_cast<int32_t>(j), a_ij);
                        a_ii += -a_ij;
                    } else {
                        a_ii += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight3(std::sqrt(r2), re_lap);
                        gx += wg * dx;
                        gy += wg * dy;
                        gz += wg * dz;
                    }
                }
            });
            double sxp, syp, szp;
            if (use_spp && spp_particle(i, re_lap, gx, gy, gz, sxp, syp, szp)) {
                const double ddx = x[i] - sxp, ddy = y[i] - syp, ddz = z[i] - szp;
                a_ii += -ppe_coefficient(std::sqrt(dot3(ddx, ddy, ddz, ddx, ddy, ddz)));
            }
            a_i.emplace_back(static_cast<int32_t>(i), a_ii);
        }
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
        const int rc = oracle_cg_solve_csr(static_cast<int64_t>(count()), row_ptr.data(), col.data(), val.data(),
                                           b.data(), xs.data(), prm.eps, prm.criterion, prm.max_cg_iters,
                                           &last_iters, &last_rr0, &last_rr);
        if (rc != MPS_OK)
            throw Oracle3Error{rc, "Conjugate Gradient method couldn't solve Pressure Poison Equation"};
    }

    /* ComputeImplicitForces (Computer.hpp:1043-1102) */
    void assign_pressure() {
        for (size_t i = 0; i < count(); i++) {
            if (type[i] == MPS_TYPE_DUMMY || type[i] == MPS_TYPE_DISABLED) continue;
            const double vv = xs[i];
            p[i] = ((vv < 0) || (!spp() && is_surface(nd[i]))) ? 0 : vv;
        }
    }
    void explicit_pressure() {
        const double c = prm.sound_speed, rho0 = prm.rho;
        for (size_t i = 0; i < count(); i++) {
            const double rho = rho0 / n0 * nd[i];
            p[i] = (rho <= rho0) ? 0 : c * c * (rho - rho0);
        }
    }

    /* Detail::InvertMatrix<3> (Computer.hpp:364-422), row-major */
    static void invert3(const double* a, double val_, double* m) {
        const double a00 = a[0], a01 = a[1], a02 = a[2], a10 = a[3], a11 = a[4], a12 = a[5];
        const double a20 = a[6], a21 = a[7], a22 = a[8];
        const double det = +a00 * a11 * a22 + a01 * a12 * a20 + a02 * a10 * a21 - a00 * a12 * a21 -
                           a01 * a10 * a22 - a02 * a11 * a20;
        if (det == 0) {
            for (int k = 0; k < 9; k++) m[k] = (k % 4 == 0) ? val_ : 0;
            return;
        }
        auto d2 = [](double pa, double pb, double pc, double pd) { return pa * pd - pb * pc; };
        m[0] = +d2(a11, a12, a21, a22) / det;
        m[1] = -d2(a10, a12, a20, a22) / det;
        m[2] = +d2(a10, a11, a20, a21) / det;
        m[3] = -d2(a01, a02, a21, a22) / det;
        m[4] = +d2(a00, a02, a20, a22) / det;
        m[5] = -d2(a00, a01, a20, a21) / det;
        m[6] = +d2(a01, a02, a11, a12) / det;
        m[7] = -d2(a00, a02, a10, a12) / det;
        m[8] = +d2(a00, a01, a10, a11) / det;
    }

    /* ModifyByPressureGradient (Computer.hpp:1433-1564), midpoint or MPS_GC */
    void pressure_gradient() {
        const size_t n = count();
        const double re2 = re * re;
        const bool use_spp = spp();
        const bool gc = flag(prm.flags, MPS_FLAG_GC);
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double C[9] = {0};
            double sxp = 0, syp = 0, szp = 0;
            bool has_spp = false;
            {
                double m[9] = {0};
                double gx = 0.0, gy = 0.0, gz = 0.0;
                for_neighbors(i, [&](size_t, double dx, double dy, double dz) {
                    const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                    if (r2 < re2) {
                        const double wg = weight3(std::sqrt(r2), re);
                        const double t_ = wg / r2;
                        const double d[3] = {dx, dy, dz};
                        for (int a = 0; a < 3; a++)
                            for (int c = 0; c < 3; c++) m[3 * a + c] += t_ * (d[a] * d[c]);
                        if (use_spp) {
                            gx += wg * dx;
                            gy += wg * dy;
                            gz += wg * dz;
                        }
                    }
                });
                has_spp = use_spp && spp_particle(i, re, gx, gy, gz, sxp, syp, szp);
                if (gc) {
                    if (has_spp) {
                        const double d[3] = {sxp - x[i], syp - y[i], szp - z[i]};
                        const double r2 = dot3(d[0], d[1], d[2], d[0], d[1], d[2]);
                        const double t_ = weight3(std::sqrt(r2), re) / r2;
                        for (int a = 0; a < 3; a++)
                            for (int c = 0; c < 3; c++) m[3 * a + c] += t_ * (d[a] * d[c]);
                    }
                    invert3(m, 3.0 / n0, C); /* InvertMatrix(invC, DIM / n0) */
                }
            }
            auto term = [&](double cc, double dx, double dy, double dz, double& sx, double& sy, double& sz) {
                if (gc) {
                    sx += cc * dot3(C[0], C[1], C[2], dx, dy, dz);
                    sy += cc * dot3(C[3], C[4], C[5], dx, dy, dz);
                    sz += cc * dot3(C[6], C[7], C[8], dx, dy, dz);
                } else {
                    sx += cc * dx;
                    sy += cc * dy;
                    sz += cc * dz;
                }
            };
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for_neighbors(i, [&](size_t j, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < re2) {
                    if (type[j] != MPS_TYPE_DUMMY) {
                        term((p[j] + p[i]) / r2 * weight3(std::sqrt(r2), re), dx, dy, dz, sx, sy, sz);
                    } else {
                        sx += 0.0;
                        sy += 0.0;
                        sz += 0.0;
                    }
                }
            });
            if (has_spp) {
                const double dx = sxp - x[i], dy = syp - y[i], dz = szp - z[i];
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                term((0.0 + p[i]) / r2 * weight3(std::sqrt(r2), re), dx, dy, dz, sx, sy, sz);
            }
            const double factor = gc ? -dt * nd[i] / (prm.rho * n0) : -dt / prm.rho * 3.0 / n0;
            dux[i] = factor * sx;
            duy[i] = factor * sy;
            duz[i] = factor * sz;
        }
        apply_du();
    }

    void apply_du() {
        for (size_t i = 0; i < count(); i++) {
            if (type[i] != MPS_TYPE_FLUID) continue;
            u[i] += dux[i];
            v[i] += duy[i];
            w[i] += duz[i];
            x[i] += dux[i] * dt;
            y[i] += duy[i] * dt;
            z[i] += duz[i] * dt;
        }
    }

    /* DynamicStabilize (Computer.hpp:1568-1656) */
    void dynamic_stabilize() {
        const size_t n = count();
        const double re2 = re * re;
        const double d = l0 - max_dx;
        const double d2 = d * d;
        const bool use_spp = spp();
        const double factor = -1.0 / (2 * dt * n0);
        ORACLE3_PARALLEL_FOR
        for (int64_t ii = 0; ii < static_cast<int64_t>(n); ii++) {
            const size_t i = static_cast<size_t>(ii);
            if (type[i] != MPS_TYPE_FLUID) continue;
            double sx = 0.0, sy = 0.0, sz = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
            for_neighbors(i, [&](size_t j, double dx, double dy, double dz) {
                const double r2 = dot3(dx, dy, dz, dx, dy, dz);
                if (r2 < re2) {
                    if (type[j] != MPS_TYPE_DUMMY && r2 < d2) {
                        const double dx0 = ox[j] - ox[i], dy0 = oy[j] - oy[i], dz0 = oz[j] - oz[i];
                        const double nrm = std::sqrt(dot3(dx0, dy0, dz0, dx0, dy0, dz0));
                        const double ex = dx0 / nrm, ey = dy0 / nrm, ez = dz0 / nrm;
                        const double r_par = dot3(dx, dy, dz, ex, ey, ez);
                        const double px = dx - r_par * ex, py = dy - r_par * ey, pz = dz - r_par * ez;
                        const double r_perp2 = dot3(px, py, pz, px, py, pz);
                        const double mag = std::sqrt(d2 - r_perp2) - r_par;
                        sx += mag * ex;
                        sy += mag * ey;
                        sz += mag * ez;
                    } else {
                        sx += 0.0;
                        sy += 0.0;
                        sz += 0.0;
                    }
                    if (use_spp) {
                        const double wg = weight3(std::sqrt(r2), re);
                        gx += wg * dx;
                        gy += wg * dy;
                        gz += wg * dz;
                    }
                }
            });
            double sxp, syp, szp;
            if (use_spp && spp_particle(i, re, gx, gy, gz, sxp, syp, szp)) {
                sx += 0.0; /* the SPP particle is excluded (Computer.hpp:1597-1598) */
                sy += 0.0;
                sz += 0.0;
            }
            dux[i] = factor * sx;
            duy[i] = factor * sy;
            duz[i] = factor * sz;
        }
        apply_du();
    }

    /* DetermineDt (Computer.hpp:759-777) */
    double determine_dt() const {
        const size_t n = count();
        if (n == 0) return max_dt;
        size_t best = 0;
        auto u2 = [&](size_t k) { return dot3(u[k], v[k], w[k], u[k], v[k], w[k]); };
        for (size_t i = 1; i < n; i++)
            if (u2(best) < u2(i)) best = i;
        const double maxU = std::sqrt(u2(best));
        if (maxU == 0) return max_dt;
        const double a = max_dx / maxU;
        return (max_dt < a) ? max_dt : a;
    }

    void begin_step(double dt_) {
        dt = dt_;
        t += dt;
    }

    /* ForwardTime (Computer.hpp:1700-1751) */
    void forward_time(double dt_) {
        if (!(dt_ > 0)) dt_ = determine_dt();
        begin_step(dt_);
        search_neighbor();
        density();
        if (flag(prm.flags, MPS_FLAG_ECS)) error_correction();
        explicit_forces();
        density();
        if (flag(prm.flags, MPS_FLAG_DS)) save_x();
        if (flag(prm.flags, MPS_FLAG_PRESSURE_EXPLICIT)) {
            explicit_pressure();
        } else {
            set_ppe();
            solve_ppe();
            assign_pressure();
        }
        pressure_gradient();
        if (flag(prm.flags, MPS_FLAG_DS)) dynamic_stabilize();
    }
};

}  // namespace

struct oracle3_handle {
    Oracle3* o;
};

namespace {
template <class F>
int guarded3(oracle3_handle* h, F f) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    try {
        f(*h->o);
        h->o->err.clear();
        return MPS_OK;
    } catch (const Oracle3Error& e) {
        h->o->err = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        h->o->err = e.what();
        return MPS_ERR_STATE;
    }
}
template <class T>
void out3(const std::vector<T>& v, T* dst) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}
template <class T>
void in3(std::vector<T>& v, const T* src) {
    if (src && !v.empty()) std::memcpy(v.data(), src, v.size() * sizeof(T));
}
}  // namespace

extern "C" {

int oracle3_create(const mps_params* prm, oracle3_handle** out) {
    if (!prm || !out) return MPS_ERR_INVALID_ARGUMENT;
    if (!(prm->l0 > 0) || !(prm->re_by_l0 > 0) || !(prm->max_y > prm->min_y)) return MPS_ERR_INVALID_ARGUMENT;
    *out = new oracle3_handle{new Oracle3(*prm)};
    return MPS_OK;
}

void oracle3_destroy(oracle3_handle* h) {
    if (!h) return;
    delete h->o;
    delete h;
}

const char* oracle3_last_error(const oracle3_handle* h) { return (h && h->o) ? h->o->err.c_str() : ""; }

int oracle3_add_particles(oracle3_handle* h, int64_t n, const int32_t* type, const double* x, const double* y,
                          const double* z, const double* u, const double* v, const double* w, const double* p,
                          const double* nd) {
    return guarded3(h, [&](Oracle3& o) {
        for (int64_t k = 0; k < n; k++) {
            o.type.push_back(type[k]);
            o.x.push_back(x[k]);
            o.y.push_back(y[k]);
            o.z.push_back(z[k]);
            o.wall_x.push_back(x[k]);
            o.wall_y.push_back(y[k]);
            o.wall_z.push_back(z[k]);
            o.u.push_back(u ? u[k] : 0.0);
            o.v.push_back(v ? v[k] : 0.0);
            o.w.push_back(w ? w[k] : 0.0);
            o.p.push_back(p ? p[k] : 0.0);
            o.nd.push_back(nd ? nd[k] : 0.0);
        }
        o.resize_aux();
    });
}

int64_t oracle3_particle_count(const oracle3_handle* h) { return (h && h->o) ? static_cast<int64_t>(h->o->count()) : -1; }

int oracle3_get_particles(const oracle3_handle* h, int32_t* type, double* x, double* y, double* z, double* u,
                          double* v, double* w, double* p, double* nd) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle3& o = *h->o;
    out3(o.type, type);
    out3(o.x, x);
    out3(o.y, y);
    out3(o.z, z);
    out3(o.u, u);
    out3(o.v, v);
    out3(o.w, w);
    out3(o.p, p);
    out3(o.nd, nd);
    return MPS_OK;
}

int oracle3_set_particles(oracle3_handle* h, const int32_t* type, const double* x, const double* y,
                          const double* z, const double* u, const double* v, const double* w, const double* p,
                          const double* nd) {
    return guarded3(h, [&](Oracle3& o) {
        in3(o.type, type);
        in3(o.x, x);
        in3(o.y, y);
        in3(o.z, z);
        in3(o.u, u);
        in3(o.v, v);
        in3(o.w, w);
        in3(o.p, p);
        in3(o.nd, nd);
    });
}

/* positionWall targets of every non-fluid particle for the next steps (Computer.hpp:1015) */
int oracle3_set_wall_positions(oracle3_handle* h, const double* wx, const double* wy, const double* wz) {
    return guarded3(h, [&](Oracle3& o) {
        in3(o.wall_x, wx);
        in3(o.wall_y, wy);
        in3(o.wall_z, wz);
    });
}

int oracle3_forward_time(oracle3_handle* h, double dt) {
    return guarded3(h, [&](Oracle3& o) { o.forward_time(dt); });
}

int oracle3_get_environment(const oracle3_handle* h, mps_environment* env) {
    if (!h || !h->o || !env) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle3& o = *h->o;
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
    env->min_y = o.prm.min_y;
    env->max_y = o.prm.max_y;
    env->grid_ny = o.gny;
    env->dim = 3;
    return MPS_OK;
}

int oracle3_stage(oracle3_handle* h, int32_t stage, double dt) {
    return guarded3(h, [&](Oracle3& o) {
        switch (stage) {
            case 0: o.begin_step(dt > 0 ? dt : o.determine_dt()); break;
            case 1: o.search_neighbor(); break;
            case 2: o.density(); break;
            case 3: o.error_correction(); break;
            case 4: o.explicit_forces(); break;
            case 5: o.save_x(); break;
            case 6: o.set_ppe(); break;
            case 7: o.solve_ppe(); break;
            case 8:
                if (flag(o.prm.flags, MPS_FLAG_PRESSURE_EXPLICIT))
                    o.explicit_pressure();
                else
                    o.assign_pressure();
                break;
            case 9: o.pressure_gradient(); break;
            case 10: o.dynamic_stabilize(); break;
            default: throw Oracle3Error{MPS_ERR_INVALID_ARGUMENT, "unknown stage"};
        }
    });
}

int oracle3_density_variation(oracle3_handle* h, double* speed) {
    return guarded3(h, [&](Oracle3& o) {
        for (size_t i = 0; i < o.count(); i++)
            speed[i] = (o.type[i] == MPS_TYPE_DUMMY || o.type[i] == MPS_TYPE_DISABLED) ? 0.0 : o.density_variation(i);
    });
}

int oracle3_get_neighbors(const oracle3_handle* h, int32_t* counts, int32_t* list, int64_t capacity, int64_t* total) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle3& o = *h->o;
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

int oracle3_get_ppe(const oracle3_handle* h, int64_t* row_ptr, int32_t* col, double* val, double* b, double* x,
                    int64_t capacity, int64_t* nnz) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle3& o = *h->o;
    const int64_t total = o.row_ptr.empty() ? 0 : o.row_ptr.back();
    if (nnz) *nnz = total;
    out3(o.row_ptr, row_ptr);
    if ((col || val) && total > capacity) return MPS_ERR_INVALID_ARGUMENT;
    out3(o.col, col);
    out3(o.val, val);
    out3(o.b, b);
    out3(o.xs, x);
    return MPS_OK;
}

int oracle3_get_aux(const oracle3_handle* h, double* n_without_spp, double* ecs, double* ox, double* oy, double* oz) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    const Oracle3& o = *h->o;
    out3(o.n_wo_spp, n_without_spp);
    out3(o.ecs, ecs);
    out3(o.ox, ox);
    out3(o.oy, oy);
    out3(o.oz, oz);
    return MPS_OK;
}

int oracle3_set_aux(oracle3_handle* h, const double* n_without_spp, const double* ecs, const double* ox,
                    const double* oy, const double* oz) {
    return guarded3(h, [&](Oracle3& o) {
        in3(o.n_wo_spp, n_without_spp);
        in3(o.ecs, ecs);
        in3(o.ox, ox);
        in3(o.oy, oy);
        in3(o.oz, oz);
    });
}

int oracle3_get_stats(const oracle3_handle* h, int32_t* cg_iterations) {
    if (!h || !h->o) return MPS_ERR_INVALID_ARGUMENT;
    if (cg_iterations) *cg_iterations = h->o->last_iters;
    return MPS_OK;
}

void oracle3_gc_invert(const double* m, double val, double* out) { Oracle3::invert3(m, val, out); }

}  // extern "C"
