"""Extract the reference's wall-hit known answers into tests/golden/hittest.npz.

Run where the reference tree exists:  python tests/golden/gen_hittest_fixture.py [REFERENCE_TREE]
(default: $PENTRACK_REFERENCE, else the build container's read-only mount).

test/HitTest/config.in fires UCN of one energy and direction from a point
1 mm in front of the inner wall of test/HollowUnitCube.STL (an aluminium
shell) for 1 ms, so each neutron meets the wall once, and
test/HitTest/showscatterdist.cxx prints the reflected, transmitted,
specularly reflected and specularly transmitted fractions of the hit log
with their expected values.  This script reads the aluminium material, the
source point, energy and direction, the simulation time and the four
expected fractions from those files as text.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    from pentrack_gb300.build import reference_tree
    tree = sys.argv[1] if len(sys.argv) > 1 else reference_tree()
    if not tree or not os.path.isdir(tree):
        sys.exit("reference tree not found: pass its path or set PENTRACK_REFERENCE")
    cfg = open(os.path.join(tree, "test", "HitTest", "config.in")).read()
    mac = open(os.path.join(tree, "test", "HitTest", "showscatterdist.cxx")).read()

    def key(name):
        return re.search(r"^\s*" + name + r"\s+([^\n#]+)", cfg, re.M).group(1).split()

    al = [float(v) for v in re.search(r"^\s*Al\s+([^\n#]+)", cfg, re.M).group(1).split()]
    expected = {}
    for label in ("Reflected", "Transmitted", "Specularly reflected", "Specularly transmitted"):
        expected[label] = float(re.search(r'"' + label + r':.*?\(Expected: ([0-9.eE+\-]+)\)', mac).group(1))
    np.savez_compressed(os.path.join(HERE, "hittest.npz"), al=np.array(al),
                        source=np.array([float(v) for v in key("parameters")]),
                        energy=float(key("Emin")[0]), phi_v=float(key("phi_v_min")[0]),
                        theta_v=float(key("theta_v_min")[0]), simtime=float(key("simtime")[0]),
                        reflected=expected["Reflected"], transmitted=expected["Transmitted"],
                        specular_reflected=expected["Specularly reflected"],
                        specular_transmitted=expected["Specularly transmitted"])
    print("HitTest fixture written:", al, expected)


if __name__ == "__main__":
    main()
