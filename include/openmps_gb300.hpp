/* openmps_gb300.hpp - C++ wrapper of the GB300 MPS time step with the reference's
 * class interface (header-only, over the C ABI of mps.h).
 *
 * Mirrors OpenMps's src/OpenMps/Particle.hpp (Particle with Type, X(), U(), P(), N(),
 * TYPE(), Disable(), W()), src/OpenMps/Environment.hpp (the constructor of :101-128,
 * whose argument list follows the method switches, and T(), Dt(), N0(), Lambda() of
 * :225-254) and src/OpenMps/Computer.hpp (Computer::Exception :1660-1666, ForwardTime
 * :1700-1751, AddParticles :1754-1777, Particles() const :1780-1783, GetEnvironment()
 * const :1786-1789, CreateComputer(allowableResidual, env, posWall, posWallPre)
 * :1800-1815), so that a caller of the reference switches by changing the include and
 * the namespace (`namespace OpenMps = openmps_gb300;`).
 *
 * The reference's compile-time method switches (MPS_HS, MPS_HL, MPS_ECS, MPS_GC, MPS_DS,
 * MPS_SPP, PRESSURE_EXPLICIT, CENTRAL_GRAVITY, DIM3) are read here as macros: they pick
 * the Environment constructor's arguments as in the reference and become the runtime
 * flags of mps_params.  openmps_gb300_defines.hpp holds the set the reference ships,
 * unless the caller included its own defines.hpp first.
 *
 * Walls: CreateComputer(eps, env, posWall, posWallPre) takes the reference's two
 * callables.  Every step the wrapper calls posWallPre(t, dt) once and posWall(i, t, dt)
 * for every particle that is not fluid (Computer.hpp:993, :1015), with t the time after
 * the step and dt the step's time step (ForwardTime() first asks the library for its
 * CFL dt, mps_determine_dt), and uploads the positions only when they changed since
 * the last upload: the reference driver's static walls (Main.cpp:311-318) cost one host
 * pass per step and no copy.  A particle that leaves the domain during a step (the
 * search disables it) takes, in that step, the wall target it already had; the next
 * step calls posWall for it like any other disabled particle.
 */
#ifndef OPENMPS_GB300_HPP
#define OPENMPS_GB300_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mps.h"
#include "openmps_gb300_defines.hpp"

namespace openmps_gb300 {

#ifdef DIM3
constexpr std::size_t DIM = 3;
constexpr std::size_t AXIS_X = 0, AXIS_Y = 1, AXIS_Z = 2;
#else
constexpr std::size_t DIM = 2;
constexpr std::size_t AXIS_X = 0, AXIS_Z = 1;
#endif
constexpr int kDim = static_cast<int>(DIM);

// The runtime method flags the caller's switches select (defines.hpp:9-56).
constexpr uint32_t kMethodFlags = 0u
#ifdef MPS_HS
                                  | MPS_FLAG_HS
#endif
#ifdef MPS_HL
                                  | MPS_FLAG_HL
#endif
#ifdef MPS_ECS
                                  | MPS_FLAG_ECS
#endif
#ifdef MPS_GC
                                  | MPS_FLAG_GC
#endif
#ifdef MPS_DS
                                  | MPS_FLAG_DS
#endif
#ifdef MPS_SPP
                                  | MPS_FLAG_SPP
#endif
#ifdef PRESSURE_EXPLICIT
                                  | MPS_FLAG_PRESSURE_EXPLICIT
#endif
#ifdef CENTRAL_GRAVITY
                                  | MPS_FLAG_CENTRAL_GRAVITY
#endif
    ;

// DIM-vector indexed like the reference's uBLAS c_vector: v(0), v(1)[, v(2)], v[i]
struct Vector {
    double v[DIM] = {};
    double& operator()(std::size_t i) { return v[i]; }
    double operator()(std::size_t i) const { return v[i]; }
    double& operator[](std::size_t i) { return v[i]; }
    double operator[](std::size_t i) const { return v[i]; }
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

// Environment(maxDt, courant, g, rho, nu, [surfaceRatio: without MPS_SPP], r_eByl_0,
// [c: PRESSURE_EXPLICIT], l_0, minX, [minY: DIM3], minZ, maxX, [maxY: DIM3], maxZ) in the
// reference's argument order (Environment.hpp:101-128).  The two-radius extension, the
// solver and the method flags are set with the members below or through mps_params.
// T(), Dt(), N0() and Lambda() are the values of the object GetEnvironment() returns
// (0 on an object the caller constructed, whose computer has not run yet).
class Environment {
public:
    mps_params params;

    // constants of the reference's Environment (derived ones refreshed by GetEnvironment)
    double MaxDt = 0, MaxDx = 0, L_0 = 0, R_e = 0, NeighborLength = 0, Rho = 0, Nu = 0;
    Vector G;

    Environment(const double maxDt, const double courant, const double g, const double rho, const double nu,
#ifndef MPS_SPP
                const double surfaceRatio,
#endif
                const double r_eByl_0,
#ifdef PRESSURE_EXPLICIT
                const double c,
#endif
                const double l_0, const double minX,
#ifdef DIM3
                const double minY,
#endif
                const double minZ, const double maxX,
#ifdef DIM3
                const double maxY,
#endif
                const double maxZ) {
        mps_default_params(&params);
        params.max_dt = maxDt;
        params.courant = courant;
        params.g = g;
        params.rho = rho;
        params.nu = nu;
#ifndef MPS_SPP
        params.surface_ratio = surfaceRatio;
#endif
        params.re_by_l0 = r_eByl_0;
#ifdef PRESSURE_EXPLICIT
        params.sound_speed = c;
#endif
        params.l0 = l_0;
        params.min_x = minX;
        params.min_z = minZ;
        params.max_x = maxX;
        params.max_z = maxZ;
#ifdef DIM3
        params.dim = 3;
        params.min_y = minY;
        params.max_y = maxY;
#endif
        params.flags = kMethodFlags;
        set_constants();
    }
    // runtime form: every field (and the method flags) from mps_params
    explicit Environment(const mps_params& p) : params(p) { set_constants(); }

    double T() const { return t_; }
    double Dt() const { return dt_; }
    double N0() const { return n0_; }
    double Lambda() const { return lambda_; }

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
    Environment& Flags(uint32_t flags) {
        params.flags = flags;
        return *this;
    }

    // the library's derived values (mps_get_environment)
    void Update(const mps_environment& e) {
        t_ = e.t;
        dt_ = e.dt;
        n0_ = e.n0;
        lambda_ = e.lambda;
        MaxDt = e.max_dt;
        MaxDx = e.max_dx;
        L_0 = e.l0;
        R_e = e.re;
        NeighborLength = e.neighbor_length;
        Rho = e.rho;
        Nu = e.nu;
    }

private:
    void set_constants() {
        MaxDt = params.max_dt;
        L_0 = params.l0;
        R_e = params.re_by_l0 * params.l0;
        Rho = params.rho;
        Nu = params.nu;
        G[AXIS_Z] = -params.g;
    }

    double t_ = 0, dt_ = 0, n0_ = 0, lambda_ = 0;
};

class Computer {
public:
    struct Exception : public std::runtime_error {
        int status;
        Exception(int code, const std::string& what) : std::runtime_error(what), status(code) {}
    };
    // positionWall(i, t, dt) and positionWallPre(t, dt) of the reference (Computer.hpp:559-562)
    using WallPosition = std::function<Vector(std::size_t, double, double)>;
    using WallPositionPre = std::function<void(double, double)>;

    // static walls: every non-fluid particle stays where it was added
    Computer(double allowableResidual, const Environment& env, int device = 0) : env_(env) {
        mps_params p = env.params;
        p.eps = allowableResidual;
        check(mps_create(&p, device, &h_), nullptr);
    }
    Computer(double allowableResidual, const Environment& env, WallPosition posWall, WallPositionPre posWallPre,
             int device = 0)
        : Computer(allowableResidual, env, device) {
        wall_ = std::move(posWall);
        wall_pre_ = std::move(posWallPre);
    }
    Computer(Computer&& o) noexcept
        : h_(o.h_), env_(std::move(o.env_)), wall_(std::move(o.wall_)), wall_pre_(std::move(o.wall_pre_)),
          types_(std::move(o.types_)), targets_(std::move(o.targets_)), disabled_seen_(o.disabled_seen_),
          types_fresh_(o.types_fresh_), cache_(std::move(o.cache_)), fresh_(o.fresh_) {
        o.h_ = nullptr;
    }
    Computer(const Computer&) = delete;
    Computer& operator=(Computer&&) noexcept = delete;
    Computer& operator=(const Computer&) = delete;
    ~Computer() {
        if (h_) mps_destroy(h_);
    }

    // ForwardTime(dt); ForwardTime() takes the CFL time step (DetermineDt)
    void ForwardTime(double dt) {
        fresh_ = false;
        if (wall_) {
            if (!(dt > 0)) check(mps_determine_dt(h_, &dt), h_);
            move_walls(dt);
        }
        check(mps_forward_time(h_, dt), h_);
    }
    void ForwardTime() { ForwardTime(-1.0); }
    // nsteps ForwardTime(dt) calls (each step still ends with its status check, so a
    // failure stops at the step that failed)
    void ForwardSteps(const double dt, int32_t nsteps) {
        if (wall_) {
            for (int32_t k = 0; k < nsteps; k++) ForwardTime(dt);
            return;
        }
        fresh_ = false;
        check(mps_forward_steps(h_, dt, nsteps), h_);
    }

    template <typename PARTICLES>
    void AddParticles(PARTICLES&& src) {
        const size_t n = src.size();
        std::vector<int32_t> t(n);
        std::vector<double> x(n), y(n), z(n), u(n), v(n), w(n), p(n), nd(n);
        size_t i = 0;
        for (const Particle& q : src) {
            t[i] = static_cast<int32_t>(q.TYPE());
            x[i] = q.X()(AXIS_X);
            z[i] = q.X()(AXIS_Z);
            u[i] = q.U()(AXIS_X);
            w[i] = q.U()(AXIS_Z);
#ifdef DIM3
            y[i] = q.X()(AXIS_Y);
            v[i] = q.U()(AXIS_Y);
#endif
            p[i] = q.P();
            nd[i] = q.N();
            i++;
        }
#ifdef DIM3
        check(mps_add_particles3(h_, static_cast<int64_t>(n), t.data(), x.data(), y.data(), z.data(), u.data(),
                                 v.data(), w.data(), p.data(), nd.data()),
              h_);
#else
        check(mps_add_particles(h_, static_cast<int64_t>(n), t.data(), x.data(), z.data(), u.data(), w.data(),
                                p.data(), nd.data()),
              h_);
#endif
        // the library's wall targets of the added particles are their positions
        types_.insert(types_.end(), t.begin(), t.end());
        targets_[0].insert(targets_[0].end(), x.begin(), x.end());
#ifdef DIM3
        targets_[1].insert(targets_[1].end(), y.begin(), y.end());
#endif
        targets_[DIM - 1].insert(targets_[DIM - 1].end(), z.begin(), z.end());
        src.clear();
        fresh_ = false;
    }

    // the particles in their original order (copied back from the device when stale)
    const std::vector<Particle>& Particles() const {
        if (fresh_) return cache_;
        const int64_t n = mps_particle_count(h_);
        std::vector<int32_t> t(n);
        std::vector<double> x(n), y(n), z(n), u(n), v(n), w(n), p(n), nd(n);
#ifdef DIM3
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
#ifdef DIM3
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

    // the environment with the current time, time step and derived constants
    const Environment& GetEnvironment() const {
        mps_environment e;
        check(mps_get_environment(h_, &e), h_);
        env_.Update(e);
        return env_;
    }
    mps_stats Stats() const {
        mps_stats s;
        check(mps_get_stats(h_, &s), h_);
        return s;
    }
    // positions of every non-fluid particle for the next steps (static from then on)
#ifdef DIM3
    void SetWallPositions(const std::vector<double>& wx, const std::vector<double>& wy,
                          const std::vector<double>& wz) {
        check(mps_set_wall_positions3(h_, wx.data(), wy.data(), wz.data()), h_);
        targets_[0] = wx;
        targets_[1] = wy;
        targets_[2] = wz;
    }
#else
    void SetWallPositions(const std::vector<double>& wx, const std::vector<double>& wz) {
        check(mps_set_wall_positions(h_, wx.data(), wz.data()), h_);
        targets_[0] = wx;
        targets_[1] = wz;
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

    // positionWallPre(t, dt) once, positionWall(i, t, dt) for every non-fluid particle
    // (Computer.hpp:993-1019, t after the step), uploaded when any target moved
    void move_walls(double dt) {
        mps_environment e;
        check(mps_get_environment(h_, &e), h_);
        const double t = e.t + dt;
        const int64_t n = mps_particle_count(h_);
        const mps_stats st = Stats();
        if (!types_fresh_ || st.disabled != disabled_seen_ || static_cast<int64_t>(types_.size()) != n) {
            types_.resize(static_cast<size_t>(n));
#ifdef DIM3
            check(mps_get_particles3(h_, types_.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                     nullptr),
                  h_);
#else
            check(mps_get_particles(h_, types_.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr), h_);
#endif
            disabled_seen_ = st.disabled;
            types_fresh_ = true;
        }
        if (wall_pre_) wall_pre_(t, dt);
        bool moved = false;
        for (int64_t i = 0; i < n; i++) {
            if (types_[static_cast<size_t>(i)] == MPS_TYPE_FLUID) continue;
            const Vector x = wall_(static_cast<std::size_t>(i), t, dt);
            for (std::size_t a = 0; a < DIM; a++) {
                double& tgt = targets_[a][static_cast<size_t>(i)];
                if (!(tgt == x(a))) {
                    tgt = x(a);
                    moved = true;
                }
            }
        }
        if (!moved) return;
#ifdef DIM3
        check(mps_set_wall_positions3(h_, targets_[0].data(), targets_[1].data(), targets_[2].data()), h_);
#else
        check(mps_set_wall_positions(h_, targets_[0].data(), targets_[1].data()), h_);
#endif
    }

    mps_handle* h_ = nullptr;
    mutable Environment env_;
    WallPosition wall_;
    WallPositionPre wall_pre_;
    std::vector<int32_t> types_;          // host copy of the particle types (wall callbacks)
    std::array<std::vector<double>, DIM> targets_;  // the wall targets last uploaded
    int32_t disabled_seen_ = -1;
    bool types_fresh_ = false;
    mutable std::vector<Particle> cache_;
    mutable bool fresh_ = false;
};

// CreateComputer(allowableResidual, env, posWall, posWallPre) (Computer.hpp:1800-1815);
// with PRESSURE_EXPLICIT there is no allowableResidual, as in the reference.
#ifndef PRESSURE_EXPLICIT
template <typename POSITION_WALL, typename POSITION_WALL_PRE>
inline Computer CreateComputer(const double allowableResidual, const Environment& env, const POSITION_WALL& posWall,
                               const POSITION_WALL_PRE& posWallPre, int device = 0) {
    return Computer(
        allowableResidual, env,
        [posWall](std::size_t i, double t, double dt) -> Vector { return posWall(i, t, dt); },
        [posWallPre](double t, double dt) { posWallPre(t, dt); }, device);
}
#else
template <typename POSITION_WALL, typename POSITION_WALL_PRE>
inline Computer CreateComputer(const Environment& env, const POSITION_WALL& posWall,
                               const POSITION_WALL_PRE& posWallPre, int device = 0) {
    return Computer(
        0.0, env, [posWall](std::size_t i, double t, double dt) -> Vector { return posWall(i, t, dt); },
        [posWallPre](double t, double dt) { posWallPre(t, dt); }, device);
}
#endif

// CreateComputer(allowableResidual, env) with static walls
inline Computer CreateComputer(double allowableResidual, const Environment& env, int device = 0) {
    return Computer(allowableResidual, env, device);
}

}  // namespace openmps_gb300

#endif /* OPENMPS_GB300_HPP */
