"""Generate the configuration fixtures tests/golden/cfg_*.npz with the oracle.

    python tests/golden/make_cfg_fixtures.py [c1 c1_lit c3 c2]

Runs the oracle (the C restatement + LAPACK through scipy) on the benchmark
configurations, at their full sizes where the CPU handles them in minutes:

  c1      plain MoM, sphere x = 2, m = 1.5 + 0.01i, a/d = 10: 4,224 cells, 12,672
          unknowns, +z incidence, V + H; S on 181 polar angles in two planes
          (Compute_EFields_MoM, src/Compute_EFields_MoM.f90:153-198,306-417);
  c1_lit  the same sphere at the literal lambda/(10|m|) cell size (489 cells);
  c3      the inhomogeneous cube of side 2 lambda truncated to 8,000 voxels
          (24,000 unknowns), 32 directions x 2 polarisations;
  c2      the CBFM benchmark scene itself: the seeded Gaussian random sphere,
          40,992 cells, 27 blocks, 24 directions x 2 polarisations, SR
          thresholding, homogeneous storage, plane-wave CBFs from the 'un' table
          (Compute_EFields_CBFME, src/Compute_EFields_CBFME.f90:221-1006).

Each fixture holds the digest of tests/golden/cfg_digest.py and the scene
signature.  The C2 run needs ~20 GB of host memory (the largest extended block
is 22.7k unknowns, solved densely as the PARDISO stand-in).  Test
infrastructure only.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import cfg_digest as D  # noqa: E402


def _save(name, wl, E, cext, cabs, S, extra=None, seconds=0.0):
    d = D.digest(E)
    out = {"signature": D.scene_signature(wl), "cext": np.asarray(cext), "cabs": np.asarray(cabs), "S": S,
           "seconds": np.array(seconds), **d}
    if extra:
        out.update(extra)
    np.savez_compressed(D.fixture_path(name), **out)
    print(f"wrote {D.fixture_path(name)}: N={E.shape[0]} ncol={E.shape[1]} ({seconds:.0f} s)", flush=True)


def mom_fixture(name, wl, rx):
    from oracle import oracle as O
    O.build()
    c = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    rth, rph = D.receivers(rx)
    t0 = time.perf_counter()
    r = O.mom_solve(c, wl["th"], wl["ph"], rth, rph)
    _save(name, wl, r["E"], r["cext"], r["cabs"], r["S"], seconds=time.perf_counter() - t0)


def cbfm_fixture(name, wl, rx):
    from oracle import oracle as O
    O.build()
    c = O.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    part = O.Partition(np.asarray(wl["offs"]), wl["ext"])
    t0 = time.perf_counter()
    r = O.cbfm_solve(c, part, wl["th"], wl["ph"], wl["niws"], homog=int(wl.get("homog", 0)))
    secs = time.perf_counter() - t0
    ce, ca = O.cext_cabs(c, wl["th"], wl["ph"], r["E"])
    rth, rph = D.receivers(rx)
    S = O.smatrix(c, rth, rph, r["E"])
    _save(name, wl, r["E"], ce, ca, S, extra={"K": np.asarray(r["K"], np.int32)}, seconds=secs)


def main(which):
    from midas_gb300 import workloads as W
    jobs = {
        "c1": lambda: mom_fixture("c1", W.mom_c1(), "polar181"),
        "c1_lit": lambda: mom_fixture("c1_lit", W.mom_tiny(), "polar181"),
        "c3": lambda: mom_fixture("c3", W.mom_c3(n_cells=8000), "grid37x2"),
        "c2": lambda: cbfm_fixture("c2", W.cbfm_c2(), "grid37x2"),
    }
    for w in which or list(jobs):
        jobs[w]()


if __name__ == "__main__":
    main(sys.argv[1:])
