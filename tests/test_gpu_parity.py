"""GPU parity: libfrico_gpu (through its C-ABI) against the CPU oracle.

Tolerances (FP64 drop-in): Z entries 1e-10 relative, input impedance,
currents and fields 1e-9 relative. Mixed precision: 1e-6 relative on Zin and
far fields after FP64 refinement.
"""
import numpy as np
import pytest

from frico_gb300 import meshes
from frico_gb300.solver import DeltaGap, PlaneWave, Simulation

pytestmark = pytest.mark.gpu

Z_TOL = 1e-10
OUT_TOL = 1e-9
MIXED_TOL = 1e-6


def rel_entrywise(a, b, floor_frac=1e-8):
    """max |a-b| / max(|b|, floor) with floor = floor_frac * max|b|."""
    b_abs = np.abs(b)
    den = np.maximum(b_abs, floor_frac * b_abs.max())
    return float((np.abs(a - b) / den).max())


def rel_norm(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def strip():
    return meshes.strip_dipole()


@pytest.fixture(scope="module")
def sphere2():
    return meshes.icosphere(2)


def oracle_for(mesh, **kw):
    from oracle import Oracle
    return Oracle(mesh, **kw)


@pytest.mark.parametrize("approx", [False, True])
def test_fill_strip(gpu_lib, strip, approx):
    o = oracle_for(strip)
    Zr = o.compute_matrix(300e6, approx=approx)
    sim = Simulation(strip, approx_matrix=approx)
    Z = sim.compute_matrix(300e6, download=True)
    assert rel_entrywise(Z, Zr) < Z_TOL
    if approx:
        assert np.abs(Z - Z.T).max() < 1e-14 * np.abs(Z).max()


@pytest.mark.parametrize("degree", [0, 2, 3, 4, 7])
def test_fill_degrees(gpu_lib, degree):
    m = meshes.icosphere(1)
    o = oracle_for(m, degree=degree)
    Zr = o.compute_matrix(450e6)
    sim = Simulation(m, degree=degree)
    Z = sim.compute_matrix(450e6, download=True)
    assert rel_entrywise(Z, Zr) < Z_TOL


def test_fill_sphere_l3(gpu_lib):
    m = meshes.icosphere(3)
    o = oracle_for(m)
    Zr = o.compute_matrix(450e6)
    sim = Simulation(m)
    Z = sim.compute_matrix(450e6, download=True)
    assert Z.shape == (1920, 1920)
    assert rel_entrywise(Z, Zr) < Z_TOL


def test_antenna_strip_fp64(gpu_lib, strip):
    f = 300e6
    o = oracle_for(strip)
    Zr = o.compute_matrix(f)
    Vr = o.rhs_delta_gap(f, [meshes.FEED_TAG])
    Ir = o.solve(Zr, Vr)
    pr = o.port_values(Ir, o.rwg(), [meshes.FEED_TAG])
    AJr, ADr, Jr = o.lump(f, Ir)
    sim = Simulation(strip)
    dg = DeltaGap((meshes.FEED_TAG,))
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, dg)
    V = sim.get_rhs()[:, 0]
    assert rel_entrywise(V, Vr) < 1e-14 if np.abs(Vr).max() > 0 else True
    I = sim.solve()[:, 0]
    assert rel_norm(I, Ir) < OUT_TOL
    pv = sim.port_values(dg)
    assert abs(pv["impedance"] - pr["impedance"]) / abs(pr["impedance"]) < OUT_TOL
    AJ, AD, J = sim.lump_currents()
    assert rel_norm(AJ, AJr) < OUT_TOL and rel_norm(AD, ADr) < OUT_TOL and rel_norm(J, Jr) < OUT_TOL
    T, P, pts = meshes.far_field_grid(10.0, 6.0)
    E, H = sim.eval_fields(pts)
    Er, Hr = o.eval_fields(pts)
    assert rel_norm(E, Er) < OUT_TOL and rel_norm(H, Hr) < OUT_TOL
    for plane in (0, 1, 2):
        G = sim.compute_gain(pv["power"].real, 10.0, plane)
        Gr = o.gain(pr["power"].real, 10.0, plane)
        assert np.max(np.abs(G - Gr) / np.abs(Gr).max()) < OUT_TOL


def test_scatter_sphere_fp64(gpu_lib, sphere2):
    f = 450e6
    o = oracle_for(sphere2)
    Zr = o.compute_matrix(f)
    Vr = o.rhs_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    Ir = o.solve(Zr, Vr)
    o.lump(f, Ir)
    sim = Simulation(sphere2)
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, PlaneWave(0.0, 0.0, 1.0, 0.0))
    assert rel_norm(sim.get_rhs()[:, 0], Vr) < 1e-13
    I = sim.solve()[:, 0]
    assert rel_norm(I, Ir) < OUT_TOL
    sig = sim.bistatic_rcs(10.0)
    sigr = o.bistatic_rcs(10.0)
    assert np.max(np.abs(sig - sigr)) / np.abs(sigr).max() < OUT_TOL
    T, P, _ = meshes.bistatic_cuts(10.0)
    s2 = sim.rcs_points(10.0, T, P)
    s2r = o.rcs(10.0, T, P)
    assert np.max(np.abs(s2 - s2r)) / np.abs(s2r).max() < OUT_TOL


def test_mixed_precision_sphere(gpu_lib):
    m = meshes.icosphere(3)
    f = 450e6
    o = oracle_for(m)
    Zr = o.compute_matrix(f)
    Vr = o.rhs_plane_wave(f, 0.0, 0.0, 1.0, 0.0)
    Ir = o.solve(Zr, Vr)
    o.lump(f, Ir)
    T, P, pts = meshes.bistatic_cuts(10.0)
    Er, _ = o.eval_fields(pts)
    sim = Simulation(m, precision="mixed")
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, PlaneWave(0.0, 0.0, 1.0, 0.0))
    I = sim.solve()[:, 0]
    st = sim.stats()
    assert st["refine_iters"] >= 1 and st["refine_residual"] < 1e-10
    assert rel_norm(I, Ir) < MIXED_TOL
    E, _ = sim.eval_fields(pts)
    assert rel_norm(E, Er) < MIXED_TOL


@pytest.mark.parametrize("pivoting,engine", [("auto", "auto"), ("none", "simt"), ("partial", "auto"),
                                             ("partial", "simt"), ("auto", "tc_f16")])
def test_mixed_pivoting_modes(gpu_lib, pivoting, engine):
    """Every complex64 factorisation strategy refines to the FP64 solution."""
    m = meshes.icosphere(3)
    f = 450e6
    o = oracle_for(m)
    Ir = o.solve(o.compute_matrix(f), o.rhs_plane_wave(f, 0.3, 0.1, 1.0, 0.5))
    sim = Simulation(m, precision="mixed", pivoting=pivoting, gemm_engine=engine)
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, PlaneWave(0.3, 0.1, 1.0, 0.5))
    I = sim.solve()[:, 0]
    st = sim.stats()
    assert st["pivoting_used"] == (1 if pivoting == "partial" else 2)
    assert 1 <= st["refine_iters"] <= 6   # complex64 factors good to ~1e-5: a few sweeps
    assert rel_norm(I, Ir) < MIXED_TOL


def test_mixed_singular_falls_back_then_reports(gpu_lib):
    """A zero pivot in the unpivoted complex64 LU triggers the partial-pivoting
    fallback; an exactly singular Z then comes back as ESINGULAR with info."""
    m = meshes.strip_dipole()
    m.vertices = m.vertices[:, [0, 2, 1]].copy()   # vertical transverse edges: zero-length RWG
    sim = Simulation(m, precision="mixed")
    sim.compute_matrix(300e6)
    sim.set_nrhs(1)
    sim.update_rhs(300e6, DeltaGap((meshes.FEED_TAG,)))
    from frico_gb300 import FricoError
    with pytest.raises(FricoError) as e:
        sim.solve()
    assert e.value.code == -2
    assert sim.stats()["pivoting_used"] == 1


@pytest.mark.parametrize("mesh,f", [("sphere3", 450e6), ("bowtie1500", 250e6), ("bowtie1500", 800e6)])
def test_double_float_fill_matches_fp64(gpu_lib, mesh, f):
    """The mixed path fills Z64 with the double-float Green table and assembly
    (FP32 pipe); the FP64 drop-in with FP64 arithmetic. Entrywise the two agree
    to 2e-13 of max |Z| (and the FP64 one stays the oracle-parity fill)."""
    m = meshes.icosphere(3) if mesh == "sphere3" else meshes.bowtie_preset(1500)
    Zd = Simulation(m, precision="mixed").compute_matrix(f, download=True)
    Z6 = Simulation(m, precision="fp64").compute_matrix(f, download=True)
    err = np.abs(Zd - Z6).max() / np.abs(Z6).max()
    assert err < 2e-13, err
    assert rel_entrywise(Zd, Z6, floor_frac=1e-6) < 1e-9


def test_double_float_fields_match_fp64(gpu_lib):
    """The mixed path evaluates fields in double-float (E, and H when asked
    for); the FP64 drop-in in FP64. On the same scatterer their E and H agree to
    1e-9 (the two solutions differ by about 1e-11), far and near."""
    m = meshes.icosphere(3)
    f = 450e6
    _, _, far = meshes.bistatic_cuts(10.0)
    rng = np.random.default_rng(7)
    d = rng.standard_normal((64, 3))
    near = d / np.linalg.norm(d, axis=1)[:, None] * rng.uniform(1.3, 3.0, (64, 1))
    out = {}
    for prec in ("mixed", "fp64"):
        sim = Simulation(m, precision=prec)
        sim.compute_matrix(f)
        sim.set_nrhs(3)
        for c, pw in enumerate([PlaneWave(0.4, 1.1, 1.0, 0.5), PlaneWave(1.3, 0.2, 0.0, 1.0), PlaneWave(2.0, 2.5, 1.0, 0.0)]):
            sim.update_rhs(f, pw, c)
        sim.solve()
        Ef, _ = sim.eval_fields(far)
        En, Hn = sim.eval_fields(near)
        Em, Hm = sim.eval_fields_multi(near)          # the multi-column pass, E and H
        Efm, _ = sim.eval_fields_multi(far, want_h=False)
        out[prec] = (Ef, En, Hn, sim.bistatic_rcs(10.0), Em, Hm, Efm)
    for a, b in zip(out["mixed"], out["fp64"]):
        assert rel_norm(a, b) < 1e-9


@pytest.mark.parametrize("nrhs", [1, 3])
def test_double_float_residual_matches_fp64(gpu_lib, nrhs):
    """The refinement residual in double-float (FP64 Z split into FP32 pairs on
    the FP32 pipe) reaches the same solution as the FP64 residual, and the
    residual it reports is the FP64 residual of the returned solution against
    the same Z (recomputed here on the host)."""
    m = meshes.icosphere(3)
    f = 450e6
    pws = [PlaneWave(0.0, 0.0, 1.0, 0.0), PlaneWave(0.7, 0.3, 0.0, 1.0), PlaneWave(1.9, 2.0, 1.0, 1.0)][:nrhs]
    out = {}
    for mode in ("auto", "fp64"):
        sim = Simulation(m, precision="mixed", residual=mode)
        Z = sim.compute_matrix(f, download=True)
        sim.set_nrhs(nrhs)
        for c, pw in enumerate(pws):
            sim.update_rhs(f, pw, c)
        B = sim.get_rhs()
        I = sim.solve()
        st = sim.stats()
        assert st["refine_residual"] <= 1e-12, (mode, st["refine_residual"])
        true = max(np.linalg.norm(B[:, c] - Z @ I[:, c]) / np.linalg.norm(B[:, c]) for c in range(nrhs))
        assert true <= 1e-12 and abs(true - st["refine_residual"]) <= 1e-13, (mode, true, st["refine_residual"])
        out[mode] = I
    assert rel_norm(out["auto"], out["fp64"]) < 1e-11


def test_mixed_strip_zin(gpu_lib, strip):
    f = 300e6
    o = oracle_for(strip)
    Zr = o.compute_matrix(f)
    Ir = o.solve(Zr, o.rhs_delta_gap(f, [meshes.FEED_TAG]))
    pr = o.port_values(Ir, o.rwg(), [meshes.FEED_TAG])
    sim = Simulation(strip, precision="mixed")
    dg = DeltaGap((meshes.FEED_TAG,))
    sim.run_context(f, dg)
    pv = sim.port_values(dg)
    assert abs(pv["impedance"] - pr["impedance"]) / abs(pr["impedance"]) < MIXED_TOL


def test_multi_rhs_and_factors(gpu_lib, sphere2):
    """Several right-hand sides share one factorisation; factors match LAPACK's solution."""
    f = 450e6
    o = oracle_for(sphere2)
    Zr = o.compute_matrix(f)
    rng = np.random.default_rng(5)
    B = rng.standard_normal((o.n, 5)) + 1j * rng.standard_normal((o.n, 5))
    Xr = o.solve(Zr, B)
    sim = Simulation(sphere2)
    sim.compute_matrix(f)
    sim.set_rhs(B)
    X = sim.solve()
    assert rel_norm(X, Xr) < OUT_TOL
    LU, ipiv = sim.get_factors()
    assert ipiv.min() >= 1 and ipiv.max() <= o.n
    L = np.tril(LU, -1) + np.eye(o.n)
    U = np.triu(LU)
    PA = Zr.copy()
    for k, p in enumerate(ipiv - 1):
        PA[[k, p]] = PA[[p, k]]
    assert rel_norm(L @ U, PA) < 1e-12


@pytest.mark.parametrize("level", [2, 3])
@pytest.mark.parametrize("engine", ["auto", "simt", "tc_f16"])
def test_mixed_unpivoted_factors(gpu_lib, level, engine):
    """The complex64 factors of the mixed path (no interchanges) reproduce Z:
    every diagonal block's LU is in place after the factorisation, whether the
    tensor-core path staged it (copied into A at the end) or the SIMT path
    wrote it directly; N = 480 ends in a 96-row block, N = 1920 in whole ones."""
    m = meshes.icosphere(level)
    f = 450e6
    Zr = oracle_for(m).compute_matrix(f)
    sim = Simulation(m, precision="mixed", pivoting="none", gemm_engine=engine)
    sim.compute_matrix(f)
    sim.set_nrhs(1)
    sim.update_rhs(f, PlaneWave(0.0, 0.0, 1.0, 0.0))
    sim.solve()
    assert sim.stats()["pivoting_used"] == 2
    LU, ipiv = sim.get_factors()
    n = Zr.shape[0]
    np.testing.assert_array_equal(ipiv, np.arange(1, n + 1))
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    # complex64 factors: FP32 rounding times the growth; the 3xFP16 updates lose the lo parts of
    # small entries (below FP16's normal range), so their factors are looser. A block left out
    # of A would give an error of order one.
    assert rel_norm(L @ U, Zr) < (1e-2 if engine == "tc_f16" else 1e-4)   # measured 1.2e-5 (tensor cores)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_set_matrix_solves_a_given_z(gpu_lib, sphere2, precision):
    """frico_gpu_set_matrix: a Z assembled elsewhere (here the oracle's) is solved
    as FRICO's solve_general solves its matrix argument; a second upload replaces
    the first (and its factors)."""
    f = 450e6
    o = oracle_for(sphere2)
    Zr = o.compute_matrix(f)
    rng = np.random.default_rng(11)
    B = rng.standard_normal((o.n, 3)) + 1j * rng.standard_normal((o.n, 3))
    Xr = np.linalg.solve(Zr, B)
    tol = OUT_TOL if precision == "fp64" else MIXED_TOL
    sim = Simulation(sphere2, precision=precision)
    sim.set_matrix(Zr, f)
    sim.set_rhs(B)
    assert rel_norm(sim.solve(), Xr) < tol
    sim.set_matrix(2.0 * Zr, f)
    sim.set_rhs(B)
    assert rel_norm(sim.solve(), 0.5 * Xr) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_set_matrix_fields_use_its_frequency(gpu_lib, sphere2, precision):
    """Fields after frico_gpu_set_matrix are evaluated at the frequency given with
    Z, as after a fill at that frequency (the lumping and the Green function of
    eval_fields take it from the context), even after a fill at another one."""
    f = 450e6
    pw = PlaneWave(0.0, 0.0, 1.0, 0.0)
    pts = meshes.sph2rect(10.0, np.linspace(0.0, np.pi, 19), np.zeros(19))
    ref = Simulation(sphere2, precision=precision)
    ref.compute_matrix(f)
    ref.update_rhs(f, pw)
    ref.solve()
    E_ref, H_ref = ref.eval_fields(pts)
    o = oracle_for(sphere2)
    sim = Simulation(sphere2, precision=precision)
    sim.compute_matrix(300e6)            # a fill at another frequency first
    sim.set_matrix(o.compute_matrix(f), f)
    sim.update_rhs(f, pw)
    sim.solve()
    E, H = sim.eval_fields(pts)
    tol = OUT_TOL if precision == "fp64" else MIXED_TOL
    assert rel_norm(E, E_ref) < tol and rel_norm(H, H_ref) < tol


def test_set_matrix_symmetric_modes_read_the_upper_triangle(gpu_lib, sphere2):
    """With force_symmetry (FRICO's -S: solve_symmetric, zsytrf uplo = 'U') the
    matrix argument's lower triangle is not read: a Z whose lower triangle is
    garbage solves as the symmetric matrix built from its upper triangle."""
    f = 450e6
    o = oracle_for(sphere2)
    Zr = o.compute_matrix(f)
    Zs = np.triu(Zr) + np.triu(Zr, 1).T
    rng = np.random.default_rng(5)
    B = rng.standard_normal((o.n, 2)) + 1j * rng.standard_normal((o.n, 2))
    Xr = np.linalg.solve(Zs, B)
    Zbad = Zr.copy()
    Zbad[np.tril_indices(o.n, -1)] = 1e3 * (1 + 1j)
    sim = Simulation(sphere2, precision="fp64", force_symmetry=True)
    sim.set_matrix(Zbad, f)
    sim.set_rhs(B)
    assert rel_norm(sim.solve(), Xr) < OUT_TOL


def test_sphere_l4_mixed_matches_fp64_at_full_size(gpu_lib):
    """The headline workload at its full size (7680 unknowns, 450 MHz, 181 x 2
    bistatic points): the mixed path's currents, far field and sigma agree with the
    FP64 drop-in's to the 1e-6 the metric requires, and its refinement reaches the
    FP64 residual tolerance."""
    m = meshes.icosphere(4)
    f = 450e6
    pw = PlaneWave(0.0, 0.0, 1.0, 0.0)
    T, P, pts = meshes.bistatic_cuts(10.0)
    out = {}
    for precision in ("fp64", "mixed"):
        sim = Simulation(m, precision=precision)
        sim.compute_matrix(f)
        sim.set_nrhs(1)
        sim.update_rhs(f, pw)
        I = sim.solve()[:, 0]
        st = sim.stats()
        E, _ = sim.eval_fields(pts)
        out[precision] = (I, E, sim.rcs_points(10.0, T, P), st)
        sim.close()
    I64, E64, s64, _ = out["fp64"]
    Imx, Emx, smx, st = out["mixed"]
    assert st["precision_used"] == 1 and st["refine_residual"] <= 1e-12
    assert rel_norm(Imx, I64) < 1e-6
    assert rel_norm(Emx, E64) < 1e-6
    assert np.max(np.abs(smx - s64)) / np.max(np.abs(s64)) < 1e-6


def test_force_symmetry(gpu_lib, strip):
    """-S (src/emw_solver.h:118-120): Z <- (Z + Z^T) / 2 before the solve, against
    the oracle's Z symmetrised the same way and LAPACK's solve_symmetric on it."""
    f = 300e6
    o = oracle_for(strip)
    Zr = o.compute_matrix(f)
    Zs = (Zr + Zr.T) / 2
    Vr = o.rhs_delta_gap(f, [meshes.FEED_TAG])
    Ir = o.solve(Zs, Vr, symmetric=True)
    sim = Simulation(strip, force_symmetry=True)
    Z = sim.compute_matrix(f, download=True)
    assert np.abs(Z - Z.T).max() == 0.0
    assert np.abs(Z - Zs).max() / np.abs(Zs).max() < 1e-10
    sim.set_nrhs(1)
    sim.update_rhs(f, DeltaGap((meshes.FEED_TAG,)))
    assert rel_norm(sim.solve()[:, 0], Ir) < OUT_TOL


def test_singular_matrix_info(gpu_lib):
    """The xy-hypot edge length makes vertical edges zero-length: Z gets zero
    rows/columns and zgetrf reports the first zero pivot; so must the GPU."""
    m = meshes.strip_dipole()
    m.vertices = m.vertices[:, [0, 2, 1]].copy()   # strip in the xz-plane: transverse edges vertical
    o = oracle_for(m)
    Zr = o.compute_matrix(300e6)
    from scipy.linalg import lapack
    _, _, info_ref = lapack.zgetrf(Zr)
    assert info_ref > 0
    sim = Simulation(m)
    sim.compute_matrix(300e6)
    sim.set_nrhs(1)
    sim.update_rhs(300e6, DeltaGap((meshes.FEED_TAG,)))
    from frico_gb300 import FricoError
    with pytest.raises(FricoError) as e:
        sim.solve()
    assert e.value.code == -2
    import ctypes
    info = ctypes.c_int32(0)
    rc = sim.lib.frico_gpu_solve(sim.ctx, None, sim.n, ctypes.byref(info))
    assert rc == -2 and info.value == info_ref


def test_true_edge_length_invariance(gpu_lib, sphere2):
    """Physical outputs do not depend on the edge-length convention."""
    f = 450e6
    out = []
    for mode in ("xy", "true"):
        sim = Simulation(sphere2, edge_length=mode)
        sim.run_context(f, PlaneWave(0.3, 0.2, 1.0, 0.0))
        out.append(sim.bistatic_rcs(10.0))
    assert np.max(np.abs(out[0] - out[1])) / np.abs(out[1]).max() < 1e-7


def test_error_paths(gpu_lib, strip):
    from frico_gb300 import FricoError
    sim = Simulation(strip)
    with pytest.raises(FricoError) as e:
        sim.solve()
    assert e.value.code == -6
    with pytest.raises(FricoError) as e:
        sim.set_options(degree=21)
    assert e.value.code == -1
    with pytest.raises(FricoError) as e:
        sim.compute_matrix(-1.0)
    assert e.value.code == -1


def test_mixed_falls_back_to_fp64_lu_when_refinement_cannot(gpu_lib, strip):
    """When neither complex64 factorisation refines to the tolerance (here forced
    by one classical sweep), the mixed solve returns the FP64 LU solution of the
    same Z and keeps those factors for further solves."""
    f = 300e6
    fp = Simulation(strip, precision="fp64")
    fp.run_context(f, DeltaGap((meshes.FEED_TAG,), 1.0))
    Ir = fp.solve()
    mx = Simulation(strip, precision="mixed", max_refine_iters=1, refine="classic")
    mx.compute_matrix(f)
    mx.set_nrhs(1)
    mx.update_rhs(f, DeltaGap((meshes.FEED_TAG,), 1.0))
    I = mx.solve()
    st = mx.stats()
    assert st["precision_used"] == 0 and st["pivoting_used"] == 1
    np.testing.assert_array_equal(I, Ir)
    I2 = mx.solve()                       # the FP64 factors stay for further right-hand sides
    np.testing.assert_array_equal(I2, Ir)


@pytest.mark.parametrize("residual", ["auto", "fp64"])
def test_mixed_ill_conditioned_refines_with_gmres(gpu_lib, residual):
    """The 1500-unknown bowtie at 250 MHz (electrically small, with skinny
    triangles at the feed) leaves kappa * eps32 close to 1 for complex64
    factors: classical refinement contracts too slowly, and the GMRES
    refinement preconditioned by the same factors reaches the FP64 solution
    without an FP64 factorisation. residual = auto: the Arnoldi products in
    double-float, fp64: in FP64; either way the returned currents' FP64
    residual (recomputed on the host) is within the bound."""
    m = meshes.bowtie_preset(1500)
    f = 250e6
    dg = DeltaGap((meshes.FEED_TAG,), 1.0)
    ref = Simulation(m, precision="fp64")
    ref.run_context(f, dg)
    Ir = ref.solve()
    mx = Simulation(m, precision="mixed", residual=residual)
    mx.delta_gap_signs = ref.delta_gap_signs
    Z = mx.compute_matrix(f, download=True)
    mx.set_nrhs(1)
    mx.update_rhs(f, dg, 0)
    B = mx.get_rhs()
    I = mx.solve()
    st = mx.stats()
    assert st["precision_used"] == 1, st
    assert st["refine_iters"] > 6, st   # GMRES, not classical refinement alone
    assert st["refine_residual"] <= 1e-12
    # At this size and frequency || |Z| |I| || / ||B|| = 1.3e4: an FP64 evaluation of the
    # residual carries noise of a few eps times that (LAPACK's own FP64 solve of this system
    # measures 1.7e-12; a 1e-16 relative change of I moves the residual by 3%), so the library's
    # FP64 residual and any other agree only to about 10% at 1e-12. Here the residual of the
    # returned currents is evaluated in extended precision and held to the tolerance plus
    # u || |Z| |I| || / ||B|| (u = eps / 2, 1.4e-12 here), the first-order noise of the FP64
    # evaluation that decided convergence.
    Zl, Il, Bl = Z.astype(np.clongdouble), I[:, 0].astype(np.clongdouble), B[:, 0].astype(np.clongdouble)
    bn = np.linalg.norm(B[:, 0])
    true = float(np.sqrt(np.sum(np.abs(Bl - Zl @ Il) ** 2))) / bn
    noise = 0.5 * np.finfo(np.float64).eps * np.linalg.norm(np.abs(Z) @ np.abs(I[:, 0])) / bn
    assert true <= 1e-12 + noise, (true, noise)
    assert rel_norm(I, Ir) < 1e-8


@pytest.mark.parametrize("profile", [False, True])
def test_mixed_factorisation_graph_replay(gpu_lib, profile):
    """The complex64 factorisation runs eagerly on the first call, is captured
    into a CUDA graph on the second and replayed after that (profiling keeps it
    eager): all three give the same currents."""
    m = meshes.icosphere(3)
    f = 450e6
    sim = Simulation(m, precision="mixed", profile_kernels=profile)
    out = []
    for _ in range(3):
        sim.compute_matrix(f)
        sim.set_nrhs(1)
        sim.update_rhs(f, PlaneWave(0.0, 0.0, 1.0, 0.0))
        out.append(sim.solve()[:, 0])
        st = sim.stats()
        assert st["pivoting_used"] == 2 and st["refine_residual"] <= 1e-12
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])
    if profile:
        assert st["gemm_launches"] > 0 and st["gemm_ms"] > 0
