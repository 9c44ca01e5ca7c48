"""Compact digests of a solved configuration, for the configuration fixtures.

The oracle's answers on the benchmark configurations are too large to commit
whole (the 40,992-cell CBFM scene has a 122,976 x 48 internal field), so each
fixture keeps a digest that the GPU answer is compared with:

  - a seeded subset of rows of E (every column): the relative error over the
    subset estimates the relative L2 error of E;
  - the column norms of E;
  - the cross sections Cext / Cabs per direction and the far-field matrix S on a
    receiver set (sums over every cell, so they see every entry of E);
  - K per block for CBFM;
  - the scene's signature (cell count, centroid sums, partition), so that a
    fixture is only compared with the scene it was made on.

Used by tests/golden/make_cfg_fixtures.py (writes), tests/test_gpu_configs.py
and bench.py (compare).  Test infrastructure: nothing in the library imports it.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
N_ROWS = 256
ROW_SEED = 4242


def fixture_path(name: str) -> str:
    return os.path.join(HERE, f"cfg_{name}.npz")


def row_subset(nrows: int, k: int = N_ROWS, seed: int = ROW_SEED) -> np.ndarray:
    """Sorted seeded row indices (all rows when nrows <= k)."""
    if nrows <= k:
        return np.arange(nrows)
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(nrows, size=k, replace=False))


def scene_signature(wl) -> np.ndarray:
    """Cell count, centroid sums and permittivity sums of a scene (+ partition sizes)."""
    xyz = np.asarray(wl["xyz"], np.float64)
    sig = [len(xyz), *xyz.sum(axis=0), float(np.abs(xyz).sum()), float(np.sum(wl["eps"]).real),
           float(np.sum(wl["eps"]).imag), float(wl["k0"]), float(wl["sc"])]
    if "offs" in wl:
        sig += [float(v) for v in wl["offs"]] + [float(len(e)) for e in wl["ext"]]
    return np.array(sig, np.float64)


def receivers(kind: str):
    """Receiver directions (degrees) of the S-matrix digest."""
    if kind == "polar181":
        th = np.concatenate([np.arange(181.0), np.arange(181.0)])
        ph = np.concatenate([np.zeros(181), np.full(181, 90.0)])
    else:   # "grid37x2"
        th = np.concatenate([np.linspace(0.0, 180.0, 37)] * 2)
        ph = np.concatenate([np.zeros(37), np.full(37, 90.0)])
    return th, ph


def digest(E: np.ndarray) -> dict:
    """E: (N, ncol) complex.  Rows subset and column norms."""
    rows = row_subset(E.shape[0])
    return {"rows": rows, "E_rows": np.ascontiguousarray(E[rows]), "colnorm": np.linalg.norm(E, axis=0)}


def compare(fx, E, cext=None, cabs=None, S=None, K=None) -> dict:
    """Relative errors of a solved configuration against a loaded fixture `fx`
    (a dict or NpzFile written by make_cfg_fixtures.py)."""
    out = {}
    rows = fx["rows"]
    Er = fx["E_rows"]
    out["E_rows_rel"] = float(np.linalg.norm(E[rows] - Er) / np.linalg.norm(Er))
    cn = np.linalg.norm(E, axis=0)
    out["colnorm_rel"] = float(np.max(np.abs(cn - fx["colnorm"]) / fx["colnorm"]))
    if cext is not None:
        out["cext_rel"] = float(np.max(np.abs(np.asarray(cext) - fx["cext"]) / np.abs(fx["cext"])))
        out["cabs_rel"] = float(np.max(np.abs(np.asarray(cabs) - fx["cabs"]) / np.abs(fx["cabs"])))
    if S is not None:
        Sr = fx["S"]
        out["S_rel"] = float(np.max(np.abs(S - Sr)) / np.max(np.abs(Sr)))
    if K is not None:
        out["K_equal"] = bool(np.array_equal(np.asarray(K), fx["K"]))
    return out
