"""A C++ caller written against the reference's Computer interface, built on openmps_gb300.hpp.

The program below makes the calls of the reference's driver in its order
(src/OpenMps/Main.cpp:291-376): it builds OpenMps::Environment with the reference's
argument list for the shipped method switches (no surfaceRatio with MPS_SPP,
Environment.hpp:101-128), keeps the initial positions in a
std::make_unique<OpenMps::Vector[]> array, passes a static-wall positionWall(i, t, dt)
and a positionWallPre(t, dt) lambda to OpenMps::CreateComputer(eps, environment,
positionWall, positionWallPre), moves the particles in with AddParticles, writes CSV
output through a template taking `const COMPUTER&` (so Particles() must be const),
steps with ForwardTime() while GetEnvironment().T() is below the next output time, and
catches decltype(computer)::Exception.  Only the include and the namespace differ
from a caller of the reference.  Its input is the reference's own Sample.xml state.

* compiled without a GPU (syntax and overloads), for 2D and with MOVING_WALL;
* on the GPU its CSV files equal the command-line driver's byte for byte;
* with MOVING_WALL, the callables move the right-hand wall; the result equals, bit for
  bit, the same steps taken through the Python binding with mps_determine_dt and
  mps_set_wall_positions, and positionWallPre runs once per step.
"""
import os
import subprocess

import numpy as np
import pytest

from openmps_gb300 import build

INCLUDE = os.path.join(build.HERE, "..", "include")

MAIN_SEQUENCE = r"""
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "openmps_gb300.hpp"  // a caller of the reference includes "Computer.hpp" here
namespace OpenMps = openmps_gb300;

namespace {

template <typename COMPUTER>
std::size_t OutputToCsv(const COMPUTER& computer, const std::size_t count) {
    char name[64];
    std::snprintf(name, sizeof(name), "result/particles_%05zu.csv", count);
    std::ofstream output(name);
    output << "Type, x, z, u, w, p, n" << std::endl;
    std::size_t alive = 0;
    for (const auto& particle : computer.Particles()) {
        output << static_cast<std::underlying_type_t<OpenMps::Particle::Type>>(particle.TYPE()) << ", "
               << particle.X()[0] << ", " << particle.X()[1] << ", " << particle.U()[0] << ", "
               << particle.U()[1] << ", " << particle.P() << ", " << particle.N() << std::endl;
        if (particle.TYPE() != OpenMps::Particle::Type::Disabled) alive++;
    }
    return alive;
}

// one particle per line: Type x z u w p n
std::vector<OpenMps::Particle> ReadParticles(std::istream& in) {
    std::vector<OpenMps::Particle> particles;
    int type;
    double x, z, u, w, p, n;
    while (in >> type >> x >> z >> u >> w >> p >> n) {
        auto particle = OpenMps::Particle(static_cast<OpenMps::Particle::Type>(type));
        particle.X()[OpenMps::AXIS_X] = x;
        particle.X()[OpenMps::AXIS_Z] = z;
        particle.U()[OpenMps::AXIS_X] = u;
        particle.U()[OpenMps::AXIS_Z] = w;
        particle.P() = p;
        particle.N() = n;
        particles.push_back(std::move(particle));
    }
    return particles;
}

}  // namespace

// argv: maxDt courant g rho nu r_eByl_0 l_0 minX minZ maxX maxZ eps endTime outputInterval
//       [wall speed, x beyond which walls move]
int main(const int argc, const char* const argv[]) {
    if (argc < 15) return 2;
    double a[16] = {};
    for (int k = 1; k < argc && k <= 16; k++) a[k - 1] = std::atof(argv[k]);
    if (std::system("mkdir -p result") != 0) return 3;
    auto&& particles = ReadParticles(std::cin);
    auto&& environment = OpenMps::Environment(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10]);
    const double eps = a[11], endTime = a[12], outputInterval = a[13];

    auto initialPosition = std::make_unique<OpenMps::Vector[]>(particles.size());
    std::transform(particles.cbegin(), particles.cend(), initialPosition.get(),
                   [](auto particle) { return particle.X(); });
#ifdef MOVING_WALL
    const double speed = a[14], xCut = a[15];
    const auto positionWall = [&initialPosition, speed, xCut](auto i, auto t, auto) {
        auto x = initialPosition[i];
        if (x[OpenMps::AXIS_X] > xCut) x[OpenMps::AXIS_X] += speed * t;
        return x;
    };
#else
    const auto positionWall = [&initialPosition](auto i, auto, auto) { return initialPosition[i]; };
#endif
    std::size_t preCalls = 0;
    const auto positionWallPre = [&preCalls](auto, auto) { preCalls++; };

    auto computer = OpenMps::CreateComputer(eps, environment, positionWall, positionWallPre);
    computer.AddParticles(std::move(particles));

    {
        const auto count = OutputToCsv(computer, 0);
        std::printf("#%05d: t=%8.4f (%05d), %12zu particles\n", 0, 0.0, 0, count);
    }
    double nextOutputT = 0;
    std::size_t iteration = 0;
    const auto endCount = static_cast<std::size_t>(std::ceil(endTime / outputInterval));
    for (auto outputCount = decltype(endCount){1}; outputCount <= endCount; outputCount++) {
        double tComputer = computer.GetEnvironment().T();
        try {
            nextOutputT += outputInterval;
            while (tComputer < nextOutputT) {
                computer.ForwardTime();
                tComputer = computer.GetEnvironment().T();
                iteration++;
            }
            const auto count = OutputToCsv(computer, outputCount);
            std::printf("#%05zu: t=%8.4f (%05zu), %12zu particles\n", outputCount, tComputer, iteration, count);
        } catch (decltype(computer)::Exception ex) {
            std::cout << "!!!!ERROR!!!!" << std::endl << ex.what() << std::endl;
            break;
        }
    }
    // the final state at full precision, for a bit-exact comparison
    FILE* f = std::fopen("final.txt", "w");
    for (const auto& particle : computer.Particles())
        std::fprintf(f, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", static_cast<int>(particle.TYPE()),
                     particle.X()[0], particle.X()[1], particle.U()[0], particle.U()[1], particle.P(), particle.N());
    std::fclose(f);
    std::printf("steps %zu positionWallPre %zu N0 %.17g\n", iteration, preCalls, computer.GetEnvironment().N0());
    std::cout << "finished" << std::endl;
    return 0;
}
"""

END_TIME = 0.01
INTERVAL = 0.005


def _sample():
    from test_reference_fixtures import sample_scene

    return sample_scene()


def _args(s, eps, speed=None, xcut=None):
    P = s.meta["params"]
    vals = [P["max_dt"], P["courant"], P["g"], P["rho"], P["nu"], P["re_by_l0"], s.l0, s.min_x, s.min_z,
            s.max_x, s.max_z, eps, END_TIME, INTERVAL]
    if speed is not None:
        vals += [speed, xcut]
    return ["%r" % float(v) for v in vals]


def _stdin(s):
    return "\n".join("%d %.17g %.17g %.17g %.17g %.17g %.17g" % (s.type[k], s.x[k], s.z[k], s.u[k], s.w[k],
                                                                 s.p[k], s.n[k]) for k in range(s.count))


def _compile(tmp_path, defines=(), syntax_only=False):
    src = tmp_path / "main_sequence.cpp"
    src.write_text(MAIN_SEQUENCE)
    # the reference's driver catches its exception by value (Main.cpp:384), as the program
    # does: -Wcatch-value would flag that line of the caller, not the wrapper
    cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-Wno-catch-value", "-I", INCLUDE, str(src),
           *defines]
    if syntax_only:
        cmd.append("-fsyntax-only")
        exe = None
    else:
        exe = tmp_path / "main_sequence"
        cmd += ["-O2", "-ffp-contract=off", "-o", str(exe), "-L", build.HERE, "-lopenmps_gb300",
                "-Wl,-rpath," + build.HERE]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.mark.parametrize("defines", [(), ("-DMOVING_WALL",)])
def test_main_sequence_compiles(tmp_path, defines):
    _compile(tmp_path, defines, syntax_only=True)


def test_explicit_pressure_signature_compiles(tmp_path):
    # with PRESSURE_EXPLICIT the reference's Environment takes c after r_eByl_0 and
    # CreateComputer takes no allowableResidual (Environment.hpp:114-117, Computer.hpp:1800-1815)
    src = tmp_path / "explicit.cpp"
    src.write_text(r"""
#define MPS_HS
#define MPS_HL
#define MPS_ECS
#define MPS_DS
#define MPS_SPP
#define PRESSURE_EXPLICIT
#define DEFINE_INCLUDED
#include "openmps_gb300.hpp"
namespace OpenMps = openmps_gb300;
int main() {
    OpenMps::Environment env(5e-4, 0.1, 9.8, 1000.0, 1e-6, 2.1, 20.0, 0.01, -0.05, -0.05, 0.85, 0.65);
    auto computer = OpenMps::CreateComputer(env, [](auto, auto, auto) { return OpenMps::Vector{}; },
                                            [](auto, auto) {});
    static_assert((OpenMps::kMethodFlags & MPS_FLAG_PRESSURE_EXPLICIT) != 0u, "switch not read");
    return computer.GetEnvironment().T() > 0.0;
}
""")
    res = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", INCLUDE,
                          str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.gpu
def test_main_sequence_matches_driver(gpu_lib, tmp_path):
    from test_driver import write_case

    s = _sample()
    eps = s.meta["params"]["eps"]
    exe = _compile(tmp_path)
    run_dir = tmp_path / "program"
    run_dir.mkdir()
    out = subprocess.run([str(exe), *_args(s, eps)], input=_stdin(s), capture_output=True, text=True,
                         cwd=run_dir, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "finished" in out.stdout and "ERROR" not in out.stdout
    drv_dir = tmp_path / "driver"
    drv_dir.mkdir()
    xml = drv_dir / "case.xml"
    write_case(xml, s, end=END_TIME, interval=INTERVAL, eps=eps,
               steps_per_output=int(round(INTERVAL / s.meta["params"]["max_dt"])))
    drv = subprocess.run([build.DRIVER, str(xml)], capture_output=True, text=True, cwd=drv_dir, timeout=600)
    assert drv.returncode == 0, drv.stdout + drv.stderr
    files = sorted(os.listdir(run_dir / "result"))
    assert files == sorted(os.listdir(drv_dir / "result")) and len(files) == 3
    for name in files:
        a = (run_dir / "result" / name).read_bytes()
        b = (drv_dir / "result" / name).read_bytes()
        assert a == b, name
    steps = int(out.stdout.split("steps ")[1].split()[0])
    pre = int(out.stdout.split("positionWallPre ")[1].split()[0])
    assert steps > 0 and pre == steps  # positionWallPre once per step
    assert float(out.stdout.split("N0 ")[1].split()[0]) == pytest.approx(9.774726, abs=5e-7)


@pytest.mark.gpu
def test_moving_wall_callables_match_binding(gpu_lib, tmp_path):
    from openmps_gb300 import _abi as abi
    from openmps_gb300.computer import Computer

    s = _sample()
    eps = s.meta["params"]["eps"]
    speed, xcut = 0.05, 0.5
    exe = _compile(tmp_path, ("-DMOVING_WALL",))
    out = subprocess.run([str(exe), *_args(s, eps, speed, xcut)], input=_stdin(s), capture_output=True, text=True,
                         cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "finished" in out.stdout and "ERROR" not in out.stdout
    got = np.loadtxt(tmp_path / "final.txt")
    steps = int(out.stdout.split("steps ")[1].split()[0])
    assert int(out.stdout.split("positionWallPre ")[1].split()[0]) == steps

    # the same steps through the Python binding: CFL dt first, then the wall targets at
    # t + dt for every non-fluid particle, then the step with that dt
    c = Computer(s.params(eps=eps))
    c.add_scene(s)
    x0, z0 = s.x.copy(), s.z.copy()
    wx, wz = x0.copy(), z0.copy()
    nxt, taken = 0.0, 0
    for _ in range(int(np.ceil(END_TIME / INTERVAL))):
        nxt += INTERVAL
        while c.environment().t < nxt:
            dt = c.determine_dt()
            t = c.environment().t + dt
            walls = c.particles()["type"] != abi.TYPE_FLUID
            moving = walls & (x0 > xcut)
            wx[walls] = x0[walls]
            wx[moving] = x0[moving] + speed * t
            wz[walls] = z0[walls]
            c.set_wall_positions(wx, wz)
            c.forward_time(dt)
            taken += 1
    assert taken == steps
    P = c.particles()
    ref = np.stack([P["type"], P["x"], P["z"], P["u"], P["w"], P["p"], P["n"]], axis=1)
    np.testing.assert_array_equal(got, ref)
    moved = (s.type != abi.TYPE_FLUID) & (x0 > xcut)
    assert moved.any() and np.all(P["x"][moved] > x0[moved])
