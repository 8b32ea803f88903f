"""Host-side mirror of FRICO's solver interface over libfrico_gpu.

FRICO's C++ surface (src/emw_solver.h:41-173, src/emw_postpro_common.h:33-37,
src/emw_ana_antenna.h:31-52, src/emw_ana_bistatic_rcs.h:28-45) becomes:

  Simulation(mesh, degree=1, approx_matrix=False, force_symmetry=False, Z0=50)
                                            simulation + config
  sim.compute_matrix(freq)                  compute_matrix / compute_matrix_approx
  sim.update_rhs(freq, DeltaGap|PlaneWave)  update_rhs(delta_gap | plane_wave)
  sim.solve()                               solve_general / solve_symmetric
  sim.run_context(freq, source)             run_context (fill, rhs, solve, lumping)
  sim.eval_fields(points)                   eval_fields(sim, ctx, point) over many points
  sim.port_values(dgap)                     compute_port_values
  sim.compute_gain(pwr, R, plane)           compute_gain
  sim.bistatic_rcs(R)                       the 359-angle loop of postpro_context
  do_sweep_antenna / do_sweep_bistatic      do_sweep(sim, antenna_analysis | bistatic_rcs_analysis)

Every numeric stage runs in the CUDA library; errors come back as FricoError
carrying FRICO_GPU_* codes (FRICO prints to stderr and returns false).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import FricoError, ptr
from .meshes import TriMesh


@dataclass
class DeltaGap:
    """src/sources.h:78-83"""
    interfaces: tuple
    voltage: complex = 1.0
    name: str = "feed"


@dataclass
class PlaneWave:
    """src/sources.h:34-75 (theta, phi in radians)"""
    theta: float
    phi: float
    Etheta: complex = 1.0
    Ephi: complex = 1.0


@dataclass
class FunctionSpace:
    rwg: np.ndarray               # RWG_DTYPE[n]
    edge_vertices: np.ndarray     # (n, 2) int64
    vertices: np.ndarray          # compacted (nv, 3)
    triangles: np.ndarray         # (nt, 3) int64
    tri_tags: np.ndarray          # (nt,)

    @property
    def n(self) -> int:
        return int(self.rwg.shape[0])


def _check(lib, code: int, ctx=None, what: str = ""):
    if code != _abi.OK:
        msg = lib.frico_gpu_last_error(ctx).decode() if ctx else what
        raise FricoError(code, msg or what)


def make_function_space(mesh: TriMesh, edge_length: str = "xy") -> FunctionSpace:
    """load_from_gmsh connectivity + make_function_space (host C++ in the library)."""
    lib = _abi.load()
    mode = _abi.EDGE_LENGTH_XY if edge_length == "xy" else _abi.EDGE_LENGTH_TRUE
    V = np.ascontiguousarray(mesh.vertices, np.float64)
    T = np.ascontiguousarray(mesh.triangles, np.int64)
    Cv = np.ascontiguousarray(mesh.curves, np.int64).reshape(-1, 2)
    Ct = np.ascontiguousarray(mesh.curve_tags, np.int32)
    nrwg = C.c_int64(0)
    nvo = C.c_int64(0)
    cap = 3 * mesh.nt // 2 + 3
    rwg = np.zeros(cap, _abi.RWG_DTYPE)
    ev = np.zeros((cap, 2), np.int64)
    vout = np.zeros_like(V)
    tout = np.zeros_like(T)
    rc = lib.frico_gpu_make_function_space(mesh.nv, ptr(V), mesh.nt, ptr(T), Cv.shape[0], ptr(Cv), ptr(Ct), mode,
                                           ptr(rwg), cap, C.byref(nrwg), ptr(ev), ptr(vout), C.byref(nvo), ptr(tout))
    _check(lib, rc, what="make_function_space")
    n = nrwg.value
    return FunctionSpace(rwg[:n].copy(), ev[:n].copy(), vout[: nvo.value].copy(), tout, mesh.tri_tags.copy())


def reorient_deltagap_edges(fs: FunctionSpace, interfaces, force: bool = False):
    """Returns the sign vector (None when FRICO would leave delta_gap_signs empty)."""
    lib = _abi.load()
    tags = np.asarray(interfaces, np.int32)
    signs = np.ones(fs.n)
    applied = C.c_int32(0)
    tt = np.ascontiguousarray(fs.tri_tags, np.int32)
    rc = lib.frico_gpu_reorient_deltagap(fs.vertices.shape[0], ptr(fs.vertices), ptr(fs.triangles), ptr(tt), fs.n,
                                         ptr(fs.rwg), ptr(fs.edge_vertices), len(tags), ptr(tags), int(force),
                                         ptr(signs), C.byref(applied))
    _check(lib, rc, what="reorient_deltagap_edges: feed edges missing or not connected")
    return signs if applied.value else None


class Simulation:
    def __init__(self, mesh: TriMesh, degree: int = 1, approx_matrix: bool = False,
                 force_symmetry: bool = False, precision: str = "fp64", Z0: float = 50.0,
                 h_phase: str = "compat", edge_length: str = "xy", device: int = 0,
                 max_refine_iters: int = 30, refine_tol: float = 1e-12, profile_kernels: bool = False,
                 gemm_engine: str = "auto", pivoting: str = "auto", refine: str = "auto",
                 residual: str = "auto", wait_limit_cycles: int = 0, fields: str = "auto"):
        self.lib = _abi.load()
        self.mesh = mesh
        self.fs = make_function_space(mesh, edge_length)
        self.opt = _abi.Options(degree, int(approx_matrix), int(force_symmetry),
                                _abi.PREC_MIXED if precision == "mixed" else _abi.PREC_FP64,
                                _abi.HPHASE_PHYSICAL if h_phase == "physical" else _abi.HPHASE_COMPAT,
                                max_refine_iters, refine_tol, Z0, int(profile_kernels),
                                {"auto": _abi.GEMM_AUTO, "simt": _abi.GEMM_SIMT, "tc": _abi.GEMM_TC,
                                 "tc_f16": _abi.GEMM_TC_F16}[gemm_engine],
                                {"auto": _abi.PIVOT_AUTO, "partial": _abi.PIVOT_PARTIAL,
                                 "none": _abi.PIVOT_NONE}[pivoting],
                                {"auto": _abi.REFINE_AUTO, "classic": _abi.REFINE_CLASSIC}[refine],
                                {"auto": _abi.RESIDUAL_AUTO, "fp64": _abi.RESIDUAL_FP64}[residual],
                                int(wait_limit_cycles),
                                {"auto": _abi.FIELDS_AUTO, "direct": _abi.FIELDS_DIRECT,
                                 "gemm": _abi.FIELDS_GEMM}[fields])
        self.ctx = C.c_void_p()
        rc = self.lib.frico_gpu_ctx_create(C.byref(self.ctx), device, C.byref(self.opt))
        _check(self.lib, rc, what="frico_gpu_ctx_create (is a CUDA device visible?)")
        fs = self.fs
        self._call("frico_gpu_set_mesh", fs.vertices.shape[0], ptr(fs.vertices), fs.triangles.shape[0],
                   ptr(fs.triangles), fs.n, ptr(fs.rwg))
        self.freq = None
        self.nrhs = 0
        self.delta_gap_signs = None

    # -- plumbing
    def _call(self, name, *args):
        rc = getattr(self.lib, name)(self.ctx, *args)
        if rc != _abi.OK:
            raise FricoError(rc, self.lib.frico_gpu_last_error(self.ctx).decode())
        return rc

    def close(self):
        if self.ctx:
            self.lib.frico_gpu_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self) -> int:
        return self.fs.n

    @property
    def nt(self) -> int:
        return int(self.fs.triangles.shape[0])

    def set_options(self, **kw):
        for k, v in kw.items():
            if k == "precision":
                v = _abi.PREC_MIXED if v == "mixed" else _abi.PREC_FP64
            setattr(self.opt, k, int(v) if k != "refine_tol" and k != "Z0" else float(v))
        self._call("frico_gpu_set_options", C.byref(self.opt))

    # -- stages
    def compute_matrix(self, freq: float, download: bool = False):
        Z = np.empty((self.n, self.n), np.complex128, order="F") if download else None
        self._call("frico_gpu_fill", float(freq), ptr(Z), self.n)
        self.freq = float(freq)
        return Z

    def set_matrix(self, Z: np.ndarray, freq: float):
        """A Z assembled elsewhere (n x n complex, at `freq` Hz) in place of
        compute_matrix; solve() then factors it, as FRICO's solve_general takes its
        matrix argument. With approx_matrix or force_symmetry only the upper
        triangle is used (solve_symmetric's zsytrf with uplo = 'U')."""
        Zf = np.asarray(Z, np.complex128, order="F")
        if Zf.shape != (self.n, self.n):
            raise ValueError(f"set_matrix: Z must be {self.n} x {self.n}")
        self._call("frico_gpu_set_matrix", float(freq), ptr(Zf), self.n)
        self.freq = float(freq)

    def set_nrhs(self, nrhs: int):
        self._call("frico_gpu_set_nrhs", int(nrhs))
        self.nrhs = int(nrhs)

    def update_rhs(self, freq: float, src, col: int = 0):
        if self.nrhs <= col:
            self.set_nrhs(col + 1)
        if isinstance(src, DeltaGap):
            tags = np.asarray(src.interfaces, np.int32)
            v = complex(src.voltage)
            signs = None if self.delta_gap_signs is None else np.ascontiguousarray(self.delta_gap_signs)
            self._call("frico_gpu_rhs_delta_gap", float(freq), col, len(tags), ptr(tags), _abi.C128(v.real, v.imag),
                       ptr(signs))
        elif isinstance(src, PlaneWave):
            a, b = complex(src.Etheta), complex(src.Ephi)
            self._call("frico_gpu_rhs_plane_wave", float(freq), col, float(src.theta), float(src.phi),
                       _abi.C128(a.real, a.imag), _abi.C128(b.real, b.imag))
        else:
            raise TypeError("source must be DeltaGap or PlaneWave")

    def get_rhs(self) -> np.ndarray:
        V = np.empty((self.n, self.nrhs), np.complex128, order="F")
        self._call("frico_gpu_get_rhs", ptr(V), self.n)
        return V

    def set_rhs(self, V: np.ndarray):
        V = np.asfortranarray(np.asarray(V, np.complex128).reshape(self.n, -1))
        self._call("frico_gpu_set_rhs", V.shape[1], ptr(V), self.n)
        self.nrhs = V.shape[1]

    def solve(self, download: bool = True):
        I = np.empty((self.n, self.nrhs), np.complex128, order="F") if download else None
        info = C.c_int32(0)
        self._call("frico_gpu_solve", ptr(I), self.n, C.byref(info))
        return I

    def get_factors(self):
        LU = np.empty((self.n, self.n), np.complex128, order="F")
        ipiv = np.empty(self.n, np.int32)
        self._call("frico_gpu_get_factors", ptr(LU), self.n, ptr(ipiv))
        return LU, ipiv

    def lump_currents(self, col: int = 0):
        AJ = np.empty((self.nt, 3), np.complex128)
        AdivJ = np.empty(self.nt, np.complex128)
        J = np.empty((self.nt, 3), np.complex128)
        self._call("frico_gpu_lump_currents", col, ptr(AJ), ptr(AdivJ), ptr(J))
        return AJ, AdivJ, J

    def eval_fields(self, points: np.ndarray, col: int = 0):
        Pt = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        E = np.empty((Pt.shape[0], 3), np.complex128)
        H = np.empty((Pt.shape[0], 3), np.complex128)
        self._call("frico_gpu_eval_fields", col, Pt.shape[0], ptr(Pt), ptr(E), ptr(H))
        return E, H

    def port_values(self, dg: DeltaGap, col: int = 0) -> dict:
        tags = np.asarray(dg.interfaces, np.int32)
        v = complex(dg.voltage)
        pv = _abi.PortValues()
        signs = None if self.delta_gap_signs is None else np.ascontiguousarray(self.delta_gap_signs)
        self._call("frico_gpu_port_values", col, len(tags), ptr(tags), _abi.C128(v.real, v.imag), ptr(signs),
                   C.byref(pv))
        c = lambda z: complex(z.re, z.im)  # noqa: E731
        return {"voltage": c(pv.voltage), "current": c(pv.current), "power": c(pv.power),
                "impedance": c(pv.impedance), "gamma": c(pv.gamma), "swr": pv.swr}

    def compute_gain(self, pwr: float, R: float, plane: int, col: int = 0) -> np.ndarray:
        G = np.empty(360)
        self._call("frico_gpu_gain", col, float(pwr), float(R), int(plane), ptr(G))
        return G

    def bistatic_rcs(self, R: float = 10.0, col: int = 0) -> np.ndarray:
        out = np.empty((359, 4))
        self._call("frico_gpu_bistatic_rcs", col, float(R), ptr(out))
        return out

    def rcs_points(self, R: float, theta, phi, col: int = 0) -> np.ndarray:
        th = np.ascontiguousarray(theta, np.float64)
        ph = np.ascontiguousarray(phi, np.float64)
        out = np.empty((th.shape[0], 2))
        self._call("frico_gpu_rcs_points", col, float(R), th.shape[0], ptr(th), ptr(ph), ptr(out))
        return out

    def eval_fields_multi(self, points, col0: int = 0, ncols: int | None = None, want_h: bool = True):
        """E, H for columns [col0, col0 + ncols): arrays (ncols, npts, 3)."""
        Pt = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        nc = self.nrhs - col0 if ncols is None else ncols
        E = np.empty((nc, Pt.shape[0], 3), np.complex128)
        H = np.empty((nc, Pt.shape[0], 3), np.complex128) if want_h else None
        self._call("frico_gpu_eval_fields_multi", col0, nc, Pt.shape[0], ptr(Pt), ptr(E), ptr(H))
        return E, H

    def rcs_points_multi(self, R: float, theta, phi, col0: int = 0, ncols: int | None = None) -> np.ndarray:
        """sigma_VV, sigma_HH for columns [col0, col0 + ncols) at the same points: (ncols, npts, 2)."""
        th = np.ascontiguousarray(theta, np.float64)
        ph = np.ascontiguousarray(phi, np.float64)
        nc = self.nrhs - col0 if ncols is None else ncols
        out = np.empty((nc, th.shape[0], 2))
        self._call("frico_gpu_rcs_points_multi", col0, nc, float(R), th.shape[0], ptr(th), ptr(ph), ptr(out))
        return out

    def monostatic_rcs(self, freq: float, theta, phi, Etheta=1.0, Ephi=1.0, R: float = 10.0) -> np.ndarray:
        """Monostatic RCS (FRICO's -m, left unimplemented there: src/main.cpp:92-93,
        src/emw_postpro_rcs.cpp:63-97): one plane-wave right-hand side per
        incidence direction (theta[c], phi[c]) in a single multi-RHS solve, and
        sigma_VV, sigma_HH (bistatic_RCS_unit_Ei) observed back along that
        direction at distance R. Returns (len(theta), 2)."""
        th = np.atleast_1d(np.asarray(theta, np.float64))
        ph = np.broadcast_to(np.asarray(phi, np.float64), th.shape).copy()
        self.compute_matrix(freq)
        self.set_nrhs(th.shape[0])
        for c in range(th.shape[0]):
            self.update_rhs(freq, PlaneWave(float(th[c]), float(ph[c]), Etheta, Ephi), c)
        self.solve(download=False)
        return np.stack([self.rcs_points(R, th[c:c + 1], ph[c:c + 1], col=c)[0] for c in range(th.shape[0])])

    def stats(self) -> dict:
        s = _abi.Stats()
        self.lib.frico_gpu_last_stats(self.ctx, C.byref(s))
        return {k: getattr(s, k) for k, _ in _abi.Stats._fields_}

    def sweep(self, freqs, dgap: DeltaGap | None = None, plane_waves=(), points=None, lanes: int = 0,
              currents: bool = False) -> dict:
        """Batched frequency sweep (frico_gpu_sweep): per frequency, the delta gap
        (if given) and then each plane wave as right-hand sides, port values of
        the delta gap, optional currents and E at `points` for every RHS.
        Frequencies run concurrently on `lanes` sub-contexts (0: chosen by the
        library)."""
        f = np.ascontiguousarray(freqs, np.float64).ravel()
        nf = f.shape[0]
        tags = np.asarray(dgap.interfaces if dgap is not None else (), np.int32)
        v = complex(dgap.voltage) if dgap is not None else 0j
        signs = None
        if dgap is not None and self.delta_gap_signs is not None:
            signs = np.ascontiguousarray(self.delta_gap_signs)
        pw = np.array([[p.theta, p.phi, complex(p.Etheta).real, complex(p.Etheta).imag,
                        complex(p.Ephi).real, complex(p.Ephi).imag] for p in plane_waves], np.float64).reshape(-1, 6)
        nrhs = (1 if dgap is not None else 0) + pw.shape[0]
        P = None if points is None else np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        npts = 0 if P is None else P.shape[0]
        port = (_abi.PortValues * nf)() if dgap is not None else None
        I = np.empty((nf, nrhs, self.n), np.complex128) if currents else None
        E = np.empty((nf, nrhs, npts, 3), np.complex128) if npts else None
        rep = _abi.SweepReport()
        self._call("frico_gpu_sweep", nf, ptr(f), len(tags), ptr(tags), _abi.C128(v.real, v.imag), ptr(signs),
                   pw.shape[0], ptr(pw), npts, ptr(P), int(lanes), port, ptr(I), ptr(E), C.byref(rep))
        c = lambda z: complex(z.re, z.im)  # noqa: E731
        ports = None
        if port is not None:
            ports = [{"voltage": c(p.voltage), "current": c(p.current), "power": c(p.power),
                      "impedance": c(p.impedance), "gamma": c(p.gamma), "swr": p.swr} for p in port]
        return {"freqs": f, "port": ports, "I": I, "E": E,
                "report": {k: getattr(rep, k) for k, _ in _abi.SweepReport._fields_}}

    def adjoint(self, freq: float, dgap: DeltaGap, P_obs, edge_length: str = "xy") -> dict:
        """Gradients of Re Zin, Im Zin and |E(P_obs)|^2 with respect to every vertex
        coordinate of the input mesh ((nv, 3) arrays in the mesh's own vertex
        numbering; unused vertices get 0) and the frequency (frico_gpu_adjoint).
        Runs the fill and solve at `freq` on this simulation's context."""
        tags = np.asarray(dgap.interfaces, np.int32)
        v = complex(dgap.voltage)
        signs = None if self.delta_gap_signs is None else np.ascontiguousarray(self.delta_gap_signs)
        P = np.ascontiguousarray(P_obs, np.float64).reshape(3)
        nvc = self.fs.vertices.shape[0]
        g = [np.zeros((nvc, 3)) for _ in range(3)]
        res = _abi.AdjointResult()
        mode = _abi.EDGE_LENGTH_XY if edge_length == "xy" else _abi.EDGE_LENGTH_TRUE
        self._call("frico_gpu_adjoint", float(freq), len(tags), ptr(tags), _abi.C128(v.real, v.imag), ptr(signs),
                   ptr(P), mode, ptr(g[0]), ptr(g[1]), ptr(g[2]), C.byref(res))
        self.freq = freq
        self.nrhs = 1
        # compacted vertex k is the k-th used vertex of the input mesh, in input order
        used = np.unique(np.asarray(self.mesh.triangles).ravel())
        full = []
        for a in g:
            f = np.zeros((self.mesh.nv, 3))
            f[used] = a
            full.append(f)
        c = lambda z: complex(z.re, z.im)  # noqa: E731
        return {"zin": c(res.zin), "E": np.array([c(res.e[a]) for a in range(3)]), "e2": res.e2,
                "grad_zin_re": full[0], "grad_zin_im": full[1], "grad_e2": full[2],
                "dzin_df": complex(res.dzin_re_df, res.dzin_im_df), "de2_df": res.de2_df}

    # -- composite, src/emw_solver.h:92-167
    def run_context(self, freq: float, src, download: bool = False):
        self.compute_matrix(freq)
        self.set_nrhs(1)
        self.update_rhs(freq, src, 0)
        I = self.solve(download=download)
        self._call("frico_gpu_lump_currents", 0, None, None, None)
        return I


@dataclass
class AntennaResult:
    frequency: float
    port: dict
    gain_XY: np.ndarray
    gain_YZ: np.ndarray
    gain_XZ: np.ndarray


def do_sweep_antenna(sim: Simulation, freqs, dgap: DeltaGap, rdiag_dist: float = 10.0,
                     force_reorient: bool = False) -> list[AntennaResult]:
    """do_sweep(sim, antenna_analysis), src/emw_ana_antenna.cpp:236-295 (no file output)."""
    sim.delta_gap_signs = reorient_deltagap_edges(sim.fs, dgap.interfaces, force_reorient)
    out = []
    for f in freqs:
        sim.run_context(f, dgap)
        pv = sim.port_values(dgap)
        pwr = pv["power"].real
        gains = [sim.compute_gain(pwr, rdiag_dist, p) for p in (_abi.GAIN_XY, _abi.GAIN_YZ, _abi.GAIN_XZ)]
        out.append(AntennaResult(float(f), pv, *gains))
    return out


@dataclass
class BistaticAnalysis:
    """src/emw_ana_bistatic_rcs.h:35-42 (angles in radians)"""
    radar_R: float = 10.0
    radar_theta: float = 0.0
    radar_phi: float = 0.0
    Etheta: float = 1.0
    Ephi: float = 1.0
    results: list = field(default_factory=list)


def do_sweep_bistatic(sim: Simulation, freqs, ana: BistaticAnalysis) -> list[np.ndarray]:
    """do_sweep(sim, bistatic_rcs_analysis), src/emw_ana_bistatic_rcs.cpp:120-151."""
    pw = PlaneWave(ana.radar_theta, ana.radar_phi, ana.Etheta, ana.Ephi)
    out = []
    for f in freqs:
        sim.run_context(f, pw)
        out.append(sim.bistatic_rcs(ana.radar_R))
    ana.results = out
    return out
