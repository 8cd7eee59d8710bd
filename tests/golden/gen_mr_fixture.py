"""Extract the reference's MicroRoughness known answers into tests/golden/steyerl_mr.npz.

Run where the reference tree exists:  python tests/golden/gen_mr_fixture.py [REFERENCE_TREE]
(default: $PENTRACK_REFERENCE, else the build container's read-only mount).

The reference's test/microroughnessTests.cpp checks MR::MRDist and MR::MRProb
against data digitised from Steyerl's paper (Z. Physik 254 (1972) 169, Figs.
2 and 3) for a copper surface: lines of constant diffuse reflection and
transmission probability in the (theta, phi) plane for 300 A neutrons at
73.5 deg incidence, and the total diffuse probability against wavelength.
This script reads the surface and beam parameters and the three data tables
from that file as text and stores them; tests/test_microroughness.py and
tests/test_gpu_microroughness.py apply the reference's tolerances to them.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def number(src, name):
    m = re.search(r"double\s+" + name + r"\s*=\s*([0-9eE.+\-]+)\s*(/\s*([0-9eE.+\-]+))?\s*(/\s*180\.\s*\*\s*pi)?;", src)
    v = float(m.group(1))
    if m.group(3):
        v /= float(m.group(3))
    if m.group(4):
        v *= np.pi / 180.0
    return v


def iso_lines(src, name):
    body = re.search(name + r"\s*=\s*\{(.*?)\};", src, re.S).group(1)
    out = []
    for level, pts in re.findall(r"\{\s*([0-9.eE+\-]+)\s*,\s*\{((?:\s*\{[^{}]*\}\s*,?)*)\}\s*\}", body):
        for a, b in re.findall(r"\{\s*([0-9.eE+\-]+)\s*,\s*([0-9.eE+\-]+)\s*\}", pts):
            out.append((float(level), float(a), float(b)))
    return np.array(out)


def main():
    from pentrack_gb300.build import reference_tree
    tree = sys.argv[1] if len(sys.argv) > 1 else reference_tree()
    if not tree or not os.path.isdir(tree):
        sys.exit("reference tree not found: pass its path or set PENTRACK_REFERENCE")
    src = open(os.path.join(tree, "test", "microroughnessTests.cpp")).read()
    total = re.search(r"steyerlTotalReflectionData\s*=\s*\{(.*?)\};", src, re.S).group(1)
    tot = np.array([(float(a), float(b)) for a, b in re.findall(r"\{\s*([0-9.eE+\-]+)\s*,\s*([0-9.eE+\-]+)\s*\}", total)])
    refl = iso_lines(src, "steyerlCopperReflectionData")
    trans = iso_lines(src, "steyerlCopperTransmissionData")
    np.savez_compressed(os.path.join(HERE, "steyerl_mr.npz"), kCu=number(src, "kCu"), bCu=number(src, "bCu"),
                        wCu=number(src, "wCu"), wavelength=number(src, "wavelength"), theta_i=number(src, "theta_i"),
                        reflection=refl, transmission=trans, total=tot)
    print(f"{len(refl)} reflection, {len(trans)} transmission and {len(tot)} total-probability points written")


if __name__ == "__main__":
    main()
