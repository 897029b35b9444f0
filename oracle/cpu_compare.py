"""Times the reference's own CPU ray caster (CollisionDetection::castRaysSoA, built from the
reference tree by ref.mk, through refcast.py) beside the oracle's BVH trace on the same rays and
cores: the primary-pass diffuse rays (one stratum per primitive, top face, seed 0) of the
1 M-triangle orchard.  Test infrastructure: it checks that the CPU baseline the bench reports
(the oracle) is not slower than the reference's own CPU code.  Needs the reference tree.

    python oracle/cpu_compare.py [threads ...]
"""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import oracle as om  # noqa: E402
import refcast  # noqa: E402
from helios_gb300 import scenes  # noqa: E402


def main(threads, nrays=300_000):
    sc = scenes.orchard(nx=20, ny=10, leaves_per_tree=5000, side=0.03, seed=0)
    t0 = time.perf_counter()
    ref = refcast.RefScene(sc.T, sc.ptype)
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    osc = om.OracleScene(sc.T, sc.ptype, sc.twosided)
    t_orc = time.perf_counter() - t0
    print(f"{sc.n} triangles; scene set-up: reference {t_ref:.2f} s, oracle {t_orc:.2f} s")
    o, d = osc.gen_rays(1, 0, 1, 1)
    o, d = o.reshape(-1, 3)[:nrays], d.reshape(-1, 3)[:nrays]
    for th in threads:
        t0 = time.perf_counter()
        ri, _ = ref.cast(o, d, threads=th)
        tr = time.perf_counter() - t0
        t0 = time.perf_counter()
        h, _, _, _ = osc.trace(o, d, mode=0, threads=th)
        to = time.perf_counter() - t0
        print(f"threads {th}: reference castRaysSoA {len(o) / tr / 1e6:.2f} M rays/s, "
              f"oracle {len(o) / to / 1e6:.2f} M rays/s; same hit {float((ri == h).mean()):.4f}")


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [1, os.cpu_count() or 1])
