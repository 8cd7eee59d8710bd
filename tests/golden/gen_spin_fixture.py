"""Generate tests/golden/adjoint_spin_100s.npz: the oracle's end states of 128
UCN of the adjoint-spin configuration (seed 1004, B0 = 1 uT + the eight l <= 2
harmonic terms, E = 1e6 V/m, specular walls, spins along x) tracked with
Bloch integration over the full 100 s, the FP64 CPU side of
tests/test_gpu_spin_long.py.

    python tests/golden/gen_spin_fixture.py [n] [simtime]
It takes a few minutes on 8 cores."""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 128
    T = float(sys.argv[2]) if len(sys.argv) > 2 else 100.0
    from oracle import pyoracle
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.adjoint_spin(n=n, simtime=T)
    t0 = time.time()
    out, st = pyoracle.Oracle(sc).integrate(params, parts, nthreads=os.cpu_count())
    wall = time.time() - t0
    np.savez_compressed(os.path.join(HERE, "adjoint_spin_100s.npz"), n=n, simtime=T, t=out.t, y=out.y, spin=out.spin,
                        stop_id=out.stop_id.astype(np.int8), n_hit=out.n_hit, spin_steps=st["spin_steps"], wall_s=wall)
    print(f"{n} UCN x {T} s in {wall:.0f} s; spin steps {st['spin_steps']}; stop IDs {np.unique(out.stop_id)}")


if __name__ == "__main__":
    main()
