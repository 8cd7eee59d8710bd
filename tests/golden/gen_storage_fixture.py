"""Generate tests/golden/field_storage_200s.npz: the oracle's end states of a
10,000-UCN subset of the field-storage workload tracked over the full 200 s
(seed 1002, ids 700,000 .. 709,999), the FP64 CPU side of the long-time
distribution test tests/test_gpu_storage_long.py.

Run on any machine with the oracle built (make -C oracle):
    python tests/golden/gen_storage_fixture.py [n] [first_id]
It takes about 25 minutes on 8 cores.  Stored per particle: end time,
end position, end polarisation (float64), stop ID, hit count, and the energy
drift (H_end - H_start)/(t_end - t_start) in eV/s with H from the oracle's own
field evaluation (H = Ekin + m g z - pol mu |B|, the Fermi potential is 0 in the
vacuum inside the cylinder)."""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, FIRST_ID, SIMTIME = 10_000, 700_000, 200.0


def total_energy(orc, t, y):
    from pentrack_gb300 import scenes
    m, c2 = scenes.M_N, scenes.C0 ** 2
    v2 = (y[3:6] ** 2).sum(0)
    B = orc.field(np.column_stack([y[0], y[1], y[2], t]))[0]
    return 0.5 * m * v2 * (1 + 0.75 * v2 / c2) + m * scenes.GRAV * y[2] - y[7] * (scenes.MU_N / scenes.ELE_E) * np.sqrt((B ** 2).sum(1))


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else N
    first = int(sys.argv[2]) if len(sys.argv) > 2 else FIRST_ID
    from oracle import pyoracle
    from pentrack_gb300 import workloads
    sc, params, parts = workloads.field_storage(n=n, simtime=SIMTIME, first_id=first)
    orc = pyoracle.Oracle(sc)
    t0 = time.time()
    out, st = orc.integrate(params, parts, nthreads=os.cpu_count())
    wall = time.time() - t0
    h0, h1 = total_energy(orc, parts.t, parts.y), total_energy(orc, out.t, out.y)
    drift = (h1 - h0) / np.maximum(out.t - parts.t, 1e-30)
    np.savez_compressed(os.path.join(HERE, "field_storage_200s.npz"), first_id=first, n=n, simtime=SIMTIME,
                        t=out.t, x=out.y[0], y=out.y[1], z=out.y[2], pol=out.y[7], stop_id=out.stop_id.astype(np.int8),
                        n_hit=out.n_hit, drift=drift, rk_accepted=st["rk_accepted"], wall_s=wall,
                        cores=os.cpu_count())
    print(f"{n} UCN x {SIMTIME} s in {wall:.0f} s on {os.cpu_count()} threads; stop IDs "
          f"{dict(zip(*np.unique(out.stop_id, return_counts=True)))}")


if __name__ == "__main__":
    main()
