"""Writes the reference's own input states as test fixtures (run in a container that
holds the reference source tree; the GPU tests only read the .npz files).

* reference_sample.npz  <- Benchmark/Sample/Sample.xml: the <condition> and
  <environment> values and the 1,323 particles of its <particles type="csv"> block
  (a 2D dam break at l0 = 0.008 m; the inputs of the reference's sample run);
* reference_particles_csv.npz <- src/OpenMps/particles.csv: 8,016 particles at
  l0 = 0.001 m (the CSV shipped beside the reference's sources).

Particle arrays keep the parsed doubles as they are.  Usage:
    python tests/golden/make_reference_fixtures.py <root of the OpenMps source tree>
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _csv_rows(lines):
    rows = [ln.replace(" ", "").replace("\t", "") for ln in lines if ln.strip()]
    header = rows[0].split(",")
    data = np.array([[float(v) for v in r.split(",")] for r in rows[1:]])
    return {k: data[:, header.index(k)] for k in ("Type", "x", "z", "u", "w", "p", "n")}


def sample_xml(path):
    text = open(path, encoding="utf-8").read()
    values = {}
    for section in ("condition", "environment"):
        body = text[text.index("<%s>" % section): text.index("</%s>" % section)]
        for tag, val in re.findall(r'<(\w+)\s+value="([^"]*)"', body):
            values["%s.%s" % (section, tag)] = float(val)
    a = text.index("<particles")
    csv = text[text.index(">", a) + 1: text.index("</particles>")]
    cols = _csv_rows(csv.splitlines())
    keys = sorted(values)
    return dict(cols, env_keys=np.array(keys), env_values=np.array([values[k] for k in keys]))


def main(ref_root):
    np.savez_compressed(os.path.join(HERE, "reference_sample.npz"),
                        **sample_xml(os.path.join(ref_root, "Benchmark", "Sample", "Sample.xml")))
    with open(os.path.join(ref_root, "src", "OpenMps", "particles.csv"), encoding="utf-8") as f:
        np.savez_compressed(os.path.join(HERE, "reference_particles_csv.npz"), **_csv_rows(f.read().splitlines()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPENMPS_REFERENCE", "."))
