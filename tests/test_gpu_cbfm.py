"""CBFM-E on the GPU against the oracle's restatement of Compute_EFields_CBFME."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(oracle, nbx, inhom, sc=0.2, seed=0):
    from midas_gb300 import geometry as G
    xyz = G.sphere_cells(2.0, sc)
    perm, offs = G.box_partition(xyz, *nbx)
    xyz = xyz[perm]
    ext = G.extend_blocks(xyz, offs, sc, sc)
    if inhom:
        rng = np.random.default_rng(seed)
        eps = rng.uniform(1.8, 2.6, len(xyz)) + 1j * rng.uniform(0.0, 0.05, len(xyz))
    else:
        eps = np.full(len(xyz), (1.5 + 0.01j) ** 2)
    return xyz, sc, eps, 2.0, offs, ext


@pytest.mark.parametrize("nbx,inhom,fill", [((2, 1, 1), False, "faithful"), ((2, 2, 1), True, "faithful"),
                                            ((2, 2, 1), True, "fast")])
def test_cbfm_matches_oracle(gpulib, oracle, nbx, inhom, fill):
    from midas_gb300 import _lib, geometry as G
    from midas_gb300.solver import Context
    xyz, sc, eps, k0, offs, ext = _case(oracle, nbx, inhom)
    th, ph = np.array([90.0, 35.0]), np.array([90.0, 120.0])
    niws = 91
    homog = 0 if inhom else 1
    cells = oracle.Cells(xyz, sc, eps, k0)
    keep = {}
    ref = oracle.cbfm_solve(cells, oracle.Partition(offs, ext), th, ph, niws, homog=homog, keep=keep)
    ref["sv"] = keep["sv"]
    cth, cph = G.transmitters_un(niws)
    mode = _lib.FILL_FAITHFUL if fill == "faithful" else _lib.FILL_FAST
    ctx = Context(fill_mode=mode, verbose=2).set_cells(xyz, sc, eps, k0)
    flags = _lib.CBFM_SR | (_lib.CBFM_HOMOG if homog else 0)
    E, K = ctx.cbfm_solve(offs, ext, cth, cph, th, ph, flags=flags)
    print("oracle fsr", keep["fsr"], "nnz", keep["nnz"])
    for b, sv in enumerate(ref["sv"]):
        print(f"oracle block {b}: sigma/sigma1:", " ".join(f"{v:.6e}" for v in sv / sv[0]))
    assert np.array_equal(K, ref["K"]), (K, ref["K"])
    rel = np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"])
    assert rel < 1e-6, rel
    assert ctx.info.k_total == int(np.sum(ref["K"]))
    ce, ca = ctx.cext_cabs(th, ph, E)
    ce_o, ca_o = oracle.cext_cabs(cells, th, ph, ref["E"])
    assert np.max(np.abs(ce - ce_o) / np.abs(ce_o)) < 1e-6
    assert np.max(np.abs(ca - ca_o) / np.abs(ca_o)) < 1e-6
    ctx.close()


@pytest.mark.parametrize("inhom", [False, True])
def test_cbfm_spherical_cbfs_match_oracle(gpulib, oracle, inhom):
    """CBFs from spherical-wave excitations (type_iws = 2/3, Incident_Field_Spherical,
    src/Compute_EFields_CBFME.f90:363-368): same K per block, field and cross sections
    within the CBFM bars."""
    from midas_gb300 import _lib, geometry as G
    from midas_gb300.solver import Context
    xyz, sc, eps, k0, offs, ext = _case(oracle, (2, 2, 1), inhom)
    th, ph = np.array([90.0, 35.0]), np.array([90.0, 120.0])
    niws = 91
    homog = 0 if inhom else 1
    cells = oracle.Cells(xyz, sc, eps, k0)
    ref = oracle.cbfm_solve(cells, oracle.Partition(offs, ext), th, ph, niws, homog=homog, spherical=True)
    cth, cph = G.transmitters_un(niws)
    ctx = Context(fill_mode=_lib.FILL_FAST).set_cells(xyz, sc, eps, k0)
    flags = _lib.CBFM_SR | _lib.CBFM_SPHERICAL | (_lib.CBFM_HOMOG if homog else 0)
    E, K = ctx.cbfm_solve(offs, ext, cth, cph, th, ph, flags=flags)
    assert np.array_equal(K, ref["K"]), (K, ref["K"])
    rel = np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"])
    assert rel < 1e-6, rel
    ce, ca = ctx.cext_cabs(th, ph, E)
    ce_o, ca_o = oracle.cext_cabs(cells, th, ph, ref["E"])
    assert np.max(np.abs(ce - ce_o) / np.abs(ce_o)) < 1e-6
    assert np.max(np.abs(ca - ca_o) / np.abs(ca_o)) < 1e-6
    ctx.close()


def test_cbfm_rejects_bad_partition(gpulib, oracle):
    from midas_gb300._lib import MidasError
    from midas_gb300 import geometry as G
    from midas_gb300.solver import Context
    xyz, sc, eps, k0, offs, ext = _case(oracle, (2, 1, 1), False)
    ctx = Context().set_cells(xyz, sc, eps, k0)
    cth, cph = G.transmitters_un(91)
    bad = offs.copy()
    bad[-1] -= 1
    with pytest.raises(MidasError) as e:
        ctx.cbfm_solve(bad, ext, cth, cph, [90.0], [90.0])
    assert e.value.status == 1
    ctx.close()


def test_cbfm_lanes_bit_identical(gpulib, oracle, monkeypatch):
    """The extended blocks run on concurrent lanes; every block is computed the same
    way whatever lane takes it, so E is bit-identical for any lane count, and with
    kernel-class profiling on (one lane)."""
    from midas_gb300 import _lib, geometry as G
    from midas_gb300.solver import Context
    xyz, sc, eps, k0, offs, ext = _case(oracle, (2, 2, 1), True)
    th, ph = np.array([90.0, 35.0]), np.array([90.0, 120.0])
    cth, cph = G.transmitters_un(91)
    ctx = Context(fill_mode=_lib.FILL_FAST).set_cells(xyz, sc, eps, k0)
    runs = []
    for lanes in ("1", "3", "6"):
        monkeypatch.setenv("MIDAS_CBFM_LANES", lanes)
        runs.append(ctx.cbfm_solve(offs, ext, cth, cph, th, ph, flags=_lib.CBFM_SR))
    ctx.profile(True)
    runs.append(ctx.cbfm_solve(offs, ext, cth, cph, th, ph, flags=_lib.CBFM_SR))
    prof = ctx.profile_query()
    ctx.profile(False)
    for E, K in runs[1:]:
        assert np.array_equal(E, runs[0][0]) and np.array_equal(K, runs[0][1])
    # the profiler saw the solve's kernels
    for k in ("gemm_trail", "gemm_panel", "gemm_solve", "gemm_prod", "resid", "diag_lu", "fill"):
        assert prof[k]["launches"] > 0 and prof[k]["ms"] > 0, k
    assert prof["gemm_trail"]["flops"] > 0 and prof["fill"]["bytes"] > 0
    ctx.close()
