/* openmps_gb300.hpp - C++ wrapper of the GB300 MPS time step with the reference's
 * class interface (header-only, over the C ABI of mps.h).
 *
 * Mirrors OpenMps's src/OpenMps/Particle.hpp (Particle with Type, X(), U(), P(), N(),
 * TYPE(), Disable(), W()), src/OpenMps/Environment.hpp:101-128 (the Environment
 * constructor arguments) and src/OpenMps/Computer.hpp (Computer::Exception :1660-1666,
 * ForwardTime :1700-1751, AddParticles :1754-1777, Particles :1780-1783,
 * GetEnvironment :1786-1789, CreateComputer :1800-1815), so that a caller of the
 * reference switches by changing the include and the namespace.  The reference's
 * compile-time method switches are runtime flags here (Environment::flags); walls are
 * static unless SetWallPositions is called (the positionWall callback of the reference).
 * With DIM3 defined (the reference's switch, defines.hpp:9-11) or OPENMPS_GB300_DIM3,
 * vectors have three components, Environment takes minY and maxY in the reference's
 * DIM3 order (Environment.hpp:101-128) and the computer is three-dimensional.
 */
#ifndef OPENMPS_GB300_HPP
#define OPENMPS_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mps.h"

namespace openmps_gb300 {

#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
constexpr int kDim = 3;
constexpr int AXIS_X = 0, AXIS_Y = 1, AXIS_Z = 2;
#else
constexpr int kDim = 2;
constexpr int AXIS_X = 0, AXIS_Z = 1;
#endif

// kDim-vector indexed like the reference's uBLAS c_vector: v(0), v(1)[, v(2)]
struct Vector {
    double v[kDim] = {};
    double& operator()(int i) { return v[i]; }
    double operator()(int i) const { return v[i]; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};

class Particle {
public:
    enum class Type { IncompressibleNewton = MPS_TYPE_FLUID, Wall = MPS_TYPE_WALL, Dummy = MPS_TYPE_DUMMY,
                      Disabled = MPS_TYPE_DISABLED };

    explicit Particle(const Type t) : type_(t) {}

    void Disable() { type_ = Type::Disabled; }
    static double W(const double r, const double r_e) { return ((0 < r) && (r < r_e)) ? (r_e / r - 1) : 0; }

    const Vector& X() const { return x_; }
    Vector& X() { return x_; }
    const Vector& U() const { return u_; }
    Vector& U() { return u_; }
    const double& P() const { return p_; }
    double& P() { return p_; }
    const double& N() const { return n_; }
    double& N() { return n_; }
    const Type& TYPE() const { return type_; }

private:
    Vector x_, u_;
    double p_ = 0.0, n_ = 0.0;
    Type type_;
};

// Environment(maxDt, courant, g, rho, nu, surfaceRatio, r_eByl_0, l_0, minX, [minY,] minZ,
// maxX, [maxY,] maxZ) in the reference's argument order; method flags, the Laplacian
// radius and the solver are members.
struct Environment {
    mps_params params;

#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
    Environment(double maxDt, double courant, double g, double rho, double nu, double surfaceRatio,
                double r_eByl_0, double l_0, double minX, double minY, double minZ, double maxX, double maxY,
                double maxZ, uint32_t flags = MPS_PRESET_REFERENCE) {
        fill(maxDt, courant, g, rho, nu, surfaceRatio, r_eByl_0, l_0, minX, minZ, maxX, maxZ, flags);
        params.dim = 3;
        params.min_y = minY;
        params.max_y = maxY;
    }
#else
    Environment(double maxDt, double courant, double g, double rho, double nu, double surfaceRatio,
                double r_eByl_0, double l_0, double minX, double minZ, double maxX, double maxZ,
                uint32_t flags = MPS_PRESET_REFERENCE) {
        fill(maxDt, courant, g, rho, nu, surfaceRatio, r_eByl_0, l_0, minX, minZ, maxX, maxZ, flags);
    }
#endif
    explicit Environment(const mps_params& p) : params(p) {}

    // two-radius extension: the Laplacian radius / l0 (0: same as r_e)
    Environment& LaplacianRadius(double re_lap_by_l0) {
        params.re_lap_by_l0 = re_lap_by_l0;
        return *this;
    }
    // Environment(..., c, ...) of PRESSURE_EXPLICIT (Environment.hpp:115-117)
    Environment& SoundSpeed(double c) {
        params.sound_speed = c;
        return *this;
    }
    Environment& Solver(int32_t solver, int32_t criterion = MPS_CRIT_INITIAL_RESIDUAL) {
        params.solver = solver;
        params.criterion = criterion;
        return *this;
    }

private:
    void fill(double maxDt, double courant, double g, double rho, double nu, double surfaceRatio, double r_eByl_0,
              double l_0, double minX, double minZ, double maxX, double maxZ, uint32_t flags) {
        mps_default_params(&params);
        params.max_dt = maxDt;
        params.courant = courant;
        params.g = g;
        params.rho = rho;
        params.nu = nu;
        params.surface_ratio = surfaceRatio;
        params.re_by_l0 = r_eByl_0;
        params.l0 = l_0;
        params.min_x = minX;
        params.min_z = minZ;
        params.max_x = maxX;
        params.max_z = maxZ;
        params.flags = flags;
    }
};

class Computer {
public:
    struct Exception : public std::runtime_error {
        int status;
        Exception(int code, const std::string& what) : std::runtime_error(what), status(code) {}
    };

    Computer(double allowableResidual, const Environment& env, int device = 0) {
        mps_params p = env.params;
        p.eps = allowableResidual;
        check(mps_create(&p, device, &h_), nullptr);
    }
    Computer(Computer&& o) noexcept : h_(o.h_), cache_(std::move(o.cache_)), fresh_(o.fresh_) { o.h_ = nullptr; }
    Computer(const Computer&) = delete;
    Computer& operator=(Computer&&) noexcept = delete;
    Computer& operator=(const Computer&) = delete;
    ~Computer() {
        if (h_) mps_destroy(h_);
    }

    // ForwardTime(dt); ForwardTime() takes the CFL time step (DetermineDt)
    void ForwardTime(const double dt) {
        fresh_ = false;
        check(mps_forward_time(h_, dt), h_);
    }
    void ForwardTime() { ForwardTime(-1.0); }
    // nsteps ForwardTime(dt) calls in one library call (each step still ends with its
    // status check, so a failure stops at the step that failed)
    void ForwardSteps(const double dt, int32_t nsteps) {
        fresh_ = false;
        check(mps_forward_steps(h_, dt, nsteps), h_);
    }

    void AddParticles(std::vector<Particle>&& src) {
        const size_t n = src.size();
        std::vector<int32_t> t(n);
        std::vector<double> x(n), y(n), z(n), u(n), v(n), w(n), p(n), nd(n);
        for (size_t i = 0; i < n; i++) {
            const Particle& q = src[i];
            t[i] = static_cast<int32_t>(q.TYPE());
            x[i] = q.X()(AXIS_X);
            z[i] = q.X()(AXIS_Z);
            u[i] = q.U()(AXIS_X);
            w[i] = q.U()(AXIS_Z);
#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
            y[i] = q.X()(AXIS_Y);
            v[i] = q.U()(AXIS_Y);
#endif
            p[i] = q.P();
            nd[i] = q.N();
        }
#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
        check(mps_add_particles3(h_, static_cast<int64_t>(n), t.data(), x.data(), y.data(), z.data(), u.data(),
                                 v.data(), w.data(), p.data(), nd.data()),
              h_);
#else
        check(mps_add_particles(h_, static_cast<int64_t>(n), t.data(), x.data(), z.data(), u.data(), w.data(),
                                p.data(), nd.data()),
              h_);
#endif
        src.clear();
        fresh_ = false;
    }

    // the particles in their original order (copied back from the device when stale)
    const std::vector<Particle>& Particles() {
        if (fresh_) return cache_;
        const int64_t n = mps_particle_count(h_);
        std::vector<int32_t> t(n);
        std::vector<double> x(n), y(n), z(n), u(n), v(n), w(n), p(n), nd(n);
#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
        check(mps_get_particles3(h_, t.data(), x.data(), y.data(), z.data(), u.data(), v.data(), w.data(), p.data(),
                                 nd.data()),
              h_);
#else
        check(mps_get_particles(h_, t.data(), x.data(), z.data(), u.data(), w.data(), p.data(), nd.data()), h_);
#endif
        cache_.clear();
        cache_.reserve(n);
        for (int64_t i = 0; i < n; i++) {
            Particle q(static_cast<Particle::Type>(t[i]));
            q.X()(AXIS_X) = x[i];
            q.X()(AXIS_Z) = z[i];
            q.U()(AXIS_X) = u[i];
            q.U()(AXIS_Z) = w[i];
#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
            q.X()(AXIS_Y) = y[i];
            q.U()(AXIS_Y) = v[i];
#endif
            q.P() = p[i];
            q.N() = nd[i];
            cache_.push_back(q);
        }
        fresh_ = true;
        return cache_;
    }

    mps_environment GetEnvironment() const {
        mps_environment e;
        check(mps_get_environment(h_, &e), h_);
        return e;
    }
    mps_stats Stats() const {
        mps_stats s;
        check(mps_get_stats(h_, &s), h_);
        return s;
    }
    // positions of every non-fluid particle for the next steps (positionWall)
#if defined(DIM3) || defined(OPENMPS_GB300_DIM3)
    void SetWallPositions(const std::vector<double>& wx, const std::vector<double>& wy,
                          const std::vector<double>& wz) {
        check(mps_set_wall_positions3(h_, wx.data(), wy.data(), wz.data()), h_);
    }
#else
    void SetWallPositions(const std::vector<double>& wx, const std::vector<double>& wz) {
        check(mps_set_wall_positions(h_, wx.data(), wz.data()), h_);
    }
#endif
    mps_handle* Handle() const { return h_; }

private:
    static void check(int rc, const mps_handle* h) {
        if (rc == MPS_OK) return;
        std::string msg = mps_status_string(rc);
        if (h) {
            const char* e = mps_last_error(h);
            if (e && *e) msg += std::string(": ") + e;
        }
        throw Exception(rc, msg);
    }

    mps_handle* h_ = nullptr;
    std::vector<Particle> cache_;
    bool fresh_ = false;
};

// CreateComputer(allowableResidual, env) with static walls
inline Computer CreateComputer(double allowableResidual, const Environment& env, int device = 0) {
    return Computer(allowableResidual, env, device);
}

}  // namespace openmps_gb300

#endif /* OPENMPS_GB300_HPP */
