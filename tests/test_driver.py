"""The command-line driver: the reference's XML/CSV input and CSV output contract.

The input is written in the reference driver's format (src/OpenMps/Main.cpp:63-274:
<condition>/<environment> value attributes, <particles type="csv"> with a Type, x, z,
u, w, p, n header); the parse check runs without a GPU, the run is compared with the
same steps taken through the Python binding of the same library.
"""
import os
import subprocess

import numpy as np
import pytest

from openmps_gb300 import _abi as abi
from openmps_gb300 import build, scenes

DRIVER = build.DRIVER


def write_case(path, scene, end=0.004, interval=0.002, eps=1e-10, steps_per_output=4, extra="",
               flags=None):
    P = dict(scene.meta["params"])
    if flags is not None:
        P["flags"] = flags
    rows = ["Type, x, z, u, w, p, n"]
    for k in range(scene.count):
        rows.append("%d, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g" % (
            scene.type[k], scene.x[k], scene.z[k], scene.u[k], scene.w[k], scene.p[k], scene.n[k]))
    env = "\n".join('    <%s value="%r" />' % (k, v) for k, v in (
        ("l_0", scene.l0), ("minStepCountPerOutput", steps_per_output), ("courant", P["courant"]),
        ("g", P["g"]), ("rho", P["rho"]), ("nu", P["nu"]), ("r_eByl_0", P["re_by_l0"]),
        ("surfaceRatio", P["surface_ratio"]), ("minX", scene.min_x), ("minZ", scene.min_z),
        ("maxX", scene.max_x), ("maxZ", scene.max_z), ("r_lapByl_0", P["re_lap_by_l0"]),
        ("flags", P["flags"])))
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n<openmps>\n  <condition>\n'
           '    <startTime value="0" />\n    <endTime value="%r" />\n    <outputInterval value="%r" />\n'
           '%s  </condition>\n  <environment>\n%s\n%s  </environment>\n'
           '  <particles type="csv">\n%s\n  </particles>\n</openmps>\n'
           % (end, interval, "" if eps is None else '    <eps value="%r" />\n' % eps, env, extra,
              "\n".join(rows)))
    with open(path, "w") as f:
        f.write(xml)


@pytest.fixture(scope="module")
def driver():
    build.build()
    return DRIVER


def test_parse_only(driver, tmp_path):
    s = scenes.config_c0()
    xml = tmp_path / "case.xml"
    write_case(xml, s, end=0.01, interval=0.005, steps_per_output=10)
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    assert "%d particles" % s.count in out.stdout
    kv = dict(item.split("=", 1) for item in out.stdout.strip().splitlines()[-1].split()
              if "=" in item and not item.startswith(("min=", "max=")))
    assert float(kv["maxDt"]) == 0.005 / 10
    assert float(kv["l_0"]) == s.l0
    assert float(kv["r_eByl_0"]) == s.meta["params"]["re_by_l0"]
    assert int(kv["flags"]) == abi.PRESET_REFERENCE
    assert float(kv["eps"]) == 1e-10


def test_parse_only_explicit_pressure(driver, tmp_path):
    # a PRESSURE_EXPLICIT input: no eps in <condition>, the sound speed c in <environment>
    # (Main.cpp:215-217, :263-265)
    s = scenes.config_c0()
    xml = tmp_path / "explicit.xml"
    flags = abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT
    write_case(xml, s, eps=None, flags=flags, extra='    <c value="27.5" />\n')
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    kv = dict(item.split("=", 1) for item in out.stdout.strip().splitlines()[-1].split()
              if "=" in item and not item.startswith(("min=", "max=")))
    assert int(kv["flags"]) == flags
    assert float(kv["c"]) == 27.5
    # without c the input is rejected, as the reference's xml.get throws
    write_case(xml, s, eps=None, flags=flags)
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode != 0


def test_rejects_bad_header(driver, tmp_path):
    s = scenes.config_c0()
    xml = tmp_path / "bad.xml"
    write_case(xml, s)
    text = xml.read_text().replace("Type, x, z, u, w, p, n", "Type, x, y, u, w, p, n")
    xml.write_text(text)
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode != 0
    assert "Illegal header item" in (out.stdout + out.stderr)


def _read_csv(path):
    with open(path) as f:
        head = f.readline().strip()
    assert head == "Type, x, z, u, w, p, n"
    return np.loadtxt(path, delimiter=",", skiprows=1)


@pytest.mark.gpu
def test_run_matches_python_binding(driver, tmp_path):
    from openmps_gb300.computer import Computer

    s = scenes.config_c0()
    xml = tmp_path / "case.xml"
    write_case(xml, s, end=0.004, interval=0.002, steps_per_output=4)
    out = subprocess.run([driver, str(xml)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "finished" in out.stdout
    files = sorted(os.listdir(tmp_path / "result"))
    assert files == ["particles_00000.csv", "particles_00001.csv", "particles_00002.csv"]
    # the same loop through the Python binding: ForwardTime() until t passes each output
    c = Computer(s.params(eps=1e-10, max_dt=0.002 / 4))
    c.add_scene(s)
    nxt = 0.0
    for k in (1, 2):
        nxt += 0.002
        while c.environment().t < nxt:
            c.forward_time()
        got = _read_csv(tmp_path / "result" / ("particles_%05d.csv" % k))
        P = c.particles()
        ref = np.stack([P["type"], P["x"], P["z"], P["u"], P["w"], P["p"], P["n"]], axis=1)
        # the driver prints six significant digits (default ostream formatting): up to half
        # a unit of the sixth digit, 5e-6 relative
        np.testing.assert_allclose(got, ref, rtol=5.01e-6, atol=1e-12)


def write_case3(path, scene, end=0.004, interval=0.002, eps=1e-10, steps_per_output=4):
    """A DIM3 input: minY/maxY in <environment>, the CSV with y and v (Main.cpp:38-50, :104-164)."""
    P = dict(scene.meta["params"])
    b = scene.bounds
    rows = ["Type, x, y, z, u, v, w, p, n"]
    for k in range(scene.count):
        rows.append("%d, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g, %.17g" % (
            scene.type[k], scene.x[k], scene.y[k], scene.z[k], scene.u[k], scene.v[k], scene.w[k], scene.p[k],
            scene.n[k]))
    env = "\n".join('    <%s value="%r" />' % (k, v) for k, v in (
        ("l_0", scene.l0), ("minStepCountPerOutput", steps_per_output), ("courant", P["courant"]),
        ("g", P["g"]), ("rho", P["rho"]), ("nu", P["nu"]), ("r_eByl_0", P["re_by_l0"]),
        ("surfaceRatio", P["surface_ratio"]), ("minX", b[0]), ("minY", b[1]), ("minZ", b[2]), ("maxX", b[3]),
        ("maxY", b[4]), ("maxZ", b[5]), ("flags", P["flags"])))
    xml = ('<?xml version="1.0" encoding="utf-8"?>\n<openmps>\n  <condition>\n'
           '    <startTime value="0" />\n    <endTime value="%r" />\n    <outputInterval value="%r" />\n'
           '    <eps value="%r" />\n  </condition>\n  <environment>\n%s\n  </environment>\n'
           '  <particles type="csv">\n%s\n  </particles>\n</openmps>\n' % (end, interval, eps, env, "\n".join(rows)))
    with open(path, "w") as f:
        f.write(xml)


def _scene3():
    s = scenes.tank3d(0.01, (5, 4, 6), (10, 6, 9))
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, re_by_l0=2.1, re_lap_by_l0=0.0)
    return s


def test_parse_only_3d(driver, tmp_path):
    s = _scene3()
    xml = tmp_path / "case3.xml"
    write_case3(xml, s)
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    assert "%d particles" % s.count in out.stdout
    kv = dict(item.split("=", 1) for item in out.stdout.strip().splitlines()[-1].split()
              if "=" in item and not item.startswith(("min=", "max=")))
    assert int(kv["dim"]) == 3
    assert float(kv["minY"]) == s.bounds[1] and float(kv["maxY"]) == s.bounds[4]
    # a 2D header in a DIM3 input misses y and v
    text = xml.read_text().replace("Type, x, y, z, u, v, w, p, n", "Type, x, z, u, w, p, n")
    xml.write_text(text)
    out = subprocess.run([driver, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode != 0


@pytest.mark.gpu
def test_run_3d_matches_python_binding(driver, tmp_path):
    from openmps_gb300.computer import Computer

    s = _scene3()
    xml = tmp_path / "case3.xml"
    write_case3(xml, s, end=0.004, interval=0.002, steps_per_output=4)
    out = subprocess.run([driver, str(xml)], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    c = Computer(s.params(eps=1e-10, max_dt=0.002 / 4))
    c.add_particles3(*s.arrays3())
    nxt = 0.0
    for k in (1, 2):
        nxt += 0.002
        while c.environment().t < nxt:
            c.forward_time()
        path = tmp_path / "result" / ("particles_%05d.csv" % k)
        with open(path) as f:
            assert f.readline().strip() == "Type, x, y, z, u, v, w, p, n"
        got = np.loadtxt(path, delimiter=",", skiprows=1)
        P = c.particles3()
        ref = np.stack([P[f] for f in ("type", "x", "y", "z", "u", "v", "w", "p", "n")], axis=1)
        np.testing.assert_allclose(got, ref, rtol=5.01e-6, atol=1e-12)


# ------------------------------------------------- the header-only C++ wrapper
CPP_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "openmps_gb300.hpp"
namespace OpenMps = openmps_gb300;  // a caller of the reference swaps its include and namespace
int main() {
    std::vector<OpenMps::Particle> ps;
    int n = 0;
    double t, x, y, z;
    while (std::scanf("%d %lf %lf %lf", &n, &x, &y, &z) == 4) {
        OpenMps::Particle q(static_cast<OpenMps::Particle::Type>(n));
        q.X()[OpenMps::AXIS_X] = x;
#ifdef DIM3
        q.X()[OpenMps::AXIS_Y] = y;
#endif
        q.X()[OpenMps::AXIS_Z] = z;
        ps.push_back(q);
    }
    // the reference's argument list with the shipped switches (MPS_SPP: no surfaceRatio)
#ifdef DIM3
    OpenMps::Environment env(5e-4, 0.1, 9.8, 1000.0, 1e-6, 2.1, 0.01, MINX, MINY, MINZ, MAXX, MAXY, MAXZ);
#else
    OpenMps::Environment env(5e-4, 0.1, 9.8, 1000.0, 1e-6, 2.1, 0.01, MINX, MINZ, MAXX, MAXZ);
#endif
    auto computer = OpenMps::CreateComputer(1e-10, env);
    computer.AddParticles(std::move(ps));
    for (int k = 0; k < 3; k++) computer.ForwardTime(5e-4);
    t = computer.GetEnvironment().T();
    std::printf("%.17g\n", t);
    for (const auto& q : computer.Particles()) {
        for (int a = 0; a < OpenMps::kDim; a++) std::printf("%.17g ", q.X()[a]);
        for (int a = 0; a < OpenMps::kDim; a++) std::printf("%.17g ", q.U()[a]);
        std::printf("%.17g %.17g\n", q.P(), q.N());
    }
    return 0;
}
"""


def _cpp_flags(dim, b):
    d = ["-DMINX=%r" % b[0], "-DMAXX=%r" % b[3 if dim == 3 else 2]]
    if dim == 3:
        d += ["-DDIM3", "-DMINY=%r" % b[1], "-DMINZ=%r" % b[2], "-DMAXY=%r" % b[4], "-DMAXZ=%r" % b[5]]
    else:
        d += ["-DMINZ=%r" % b[1], "-DMAXZ=%r" % b[3]]
    return d


@pytest.mark.parametrize("dim", [2, 3])
def test_cpp_wrapper_compiles(tmp_path, dim):
    src = tmp_path / "prog.cpp"
    src.write_text(CPP_PROGRAM)
    res = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                          "-I", os.path.join(build.HERE, "..", "include"), str(src)]
                         + _cpp_flags(dim, (0.0, 0.0, 0.0, 1.0, 1.0, 1.0)), capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.gpu
def test_cpp_wrapper_dim3_run(driver, tmp_path):
    # the wrapper compiled with the reference's DIM3 switch, against the Python binding
    from openmps_gb300.computer import Computer

    s = _scene3()
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, re_by_l0=2.1, re_lap_by_l0=0.0, rho=1000.0, nu=1e-6,
                            surface_ratio=0.97, courant=0.1, g=9.8, max_dt=5e-4, eps=1e-10)
    src = tmp_path / "prog.cpp"
    src.write_text(CPP_PROGRAM)
    exe = tmp_path / "prog"
    res = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                          os.path.join(build.HERE, "..", "include"), str(src), "-o", str(exe), "-L", build.HERE,
                          "-lopenmps_gb300", "-Wl,-rpath," + build.HERE] + _cpp_flags(3, s.bounds),
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    stdin = "\n".join("%d %.17g %.17g %.17g" % (s.type[k], s.x[k], s.y[k], s.z[k]) for k in range(s.count))
    out = subprocess.run([str(exe)], input=stdin, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:]])
    c = Computer(s.params())
    c.add_particles3(*s.arrays3())
    for _ in range(3):
        c.forward_time(5e-4)
    assert float(lines[0]) == c.environment().t
    P = c.particles3()
    ref = np.stack([P[f] for f in ("x", "y", "z", "u", "v", "w", "p", "n")], axis=1)
    np.testing.assert_array_equal(got, ref)
