"""Write sphere192_fp64_history.npy: the oracle's residual history of the
192^3 sphere (D = 1 in [-10, 10]^3, M = 0.5, JST scalar, 5-stage RK, CFL 2.8,
IRS 0.6, 4-level W-cycle, FMG with 50 cycles on each coarse level) in the
plain FP64 form, every cycle of the first 700 (150 FMG cycles, then 550 on
the 192^3 level), run past the point where the residual stops falling and
settles into a periodic orbit.

The oracle takes about 2 to 3 hours for it on 8 host threads, so the GPU test
compares against this file instead of running the oracle.

    python tests/golden/make_sphere192_history.py [threads]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

from code_mge_gb300 import cases as K  # noqa: E402
from oracle import oracle as O  # noqa: E402

CYCLES = 700


def case():
    c = K.sphere_box(n=192, nlevel=4, extent=10.0, mach=0.5, mgtype=2, mcyc_fine=400, smoo=0.6)
    c.prm.conv_drop = 1e30  # run every cycle
    c.prm.mcyc[3] = 100000  # 50 cycles on each coarse FMG level, then the finest until CYCLES
    return c


if __name__ == "__main__":
    O.set_threads(int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1))
    o = O.OracleCycle(case())
    hist, n, f = o.solve(max_cycles_total=CYCLES, hist_len=CYCLES)
    o.close()
    assert n == CYCLES, n
    np.save(os.path.join(HERE, "sphere192_fp64_history.npy"), hist)
    print("cycles %d, drop %.3g, cd %.12g" % (n, hist[0] / hist.min(), f.cd))
