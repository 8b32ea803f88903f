"""CPU oracle for FRICO's MoM hot path -- TEST INFRASTRUCTURE ONLY.

Wraps oracle/_build/libfrico_oracle.so (a line-by-line C++ restatement of
FRICO's fill / RHS / lumping / field code, see frico_oracle.cpp) and performs
the dense solve with the LAPACK routines FRICO calls (zgetrf/zgetrs, or
zsytrf/zsytrs for -A / -S, src/lapack_wrappers.cpp:53-177) through scipy.
Only tests, the smoke check and the CPU-baseline leg of bench.py use it.

Parity pin: the restatement's quadrature, RWG table, Z, V, I, lumped currents
and fields are compared with FRICO's own sources compiled in place
(oracle/ref/, outputs in oracle/_ref/) and with golden vectors generated from
that build (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import build as _build  # noqa: E402

_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
        sig = {
            "oracle_create": ([], vp), "oracle_destroy": ([vp], None),
            "oracle_set_degree": ([vp, i32, i32], None),
            "oracle_set_mesh": ([vp, i64, vp, i64, vp, vp, i64, vp, vp, i32], i64),
            "oracle_get_rwg": ([vp, vp], None),
            "oracle_dunavant": ([i32, vp, vp, vp, vp], i32),
            "oracle_compute_matrix": ([vp, d, vp], None),
            "oracle_compute_matrix_cols": ([vp, d, i64, i64, vp], None),
            "oracle_compute_matrix_magnitudes": ([vp, d, i64, i64, vp], None),
            "oracle_compute_matrix_approx": ([vp, d, vp], None),
            "oracle_reorient": ([vp, i32, vp, i32, vp], i32),
            "oracle_rhs_delta_gap": ([vp, d, i32, vp, d, d, vp, vp], None),
            "oracle_rhs_plane_wave": ([vp, d, d, d, d, d, d, d, vp], None),
            "oracle_lump": ([vp, d, vp, vp, vp, vp], None),
            "oracle_eval_fields": ([vp, i64, vp, vp, vp], None),
            "oracle_num_rwg": ([vp], i64), "oracle_num_tri": ([vp], i64),
        }
        for name, (args, res) in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def dunavant(degree: int, p0, p1, p2) -> np.ndarray:
    lib = _load()
    out = np.zeros((100, 4))
    a, b, c = (np.ascontiguousarray(x, np.float64) for x in (p0, p1, p2))
    k = lib.oracle_dunavant(degree, _p(a), _p(b), _p(c), _p(out))
    return out[:k].copy()


class Oracle:
    """FRICO `simulation` restated on the CPU for one mesh."""

    def __init__(self, mesh, degree: int = 1, edge_length: str = "xy", h_phase: str = "compat"):
        self.lib = _load()
        self.s = self.lib.oracle_create()
        self.lib.oracle_set_degree(self.s, degree, int(h_phase == "physical"))
        V = np.ascontiguousarray(mesh.vertices, np.float64)
        T = np.ascontiguousarray(mesh.triangles, np.int64)
        tg = np.ascontiguousarray(mesh.tri_tags, np.int32)
        Cv = np.ascontiguousarray(mesh.curves, np.int64).reshape(-1, 2)
        Ct = np.ascontiguousarray(mesh.curve_tags, np.int32)
        n = self.lib.oracle_set_mesh(self.s, V.shape[0], _p(V), T.shape[0], _p(T), _p(tg), Cv.shape[0], _p(Cv),
                                     _p(Ct), int(edge_length == "xy"))
        if n < 0:
            raise ValueError({-1: "multiple_triangles", -2: "lonely_edge"}[n])
        self.n = int(n)
        self.nt = int(self.lib.oracle_num_tri(self.s))
        self.degree = degree
        self.freq = None

    def __del__(self):
        try:
            self.lib.oracle_destroy(self.s)
        except Exception:
            pass

    def rwg(self) -> np.ndarray:
        out = np.zeros((self.n, 17))
        self.lib.oracle_get_rwg(self.s, _p(out))
        return out

    def compute_matrix(self, freq: float, approx: bool = False) -> np.ndarray:
        Z = np.zeros((self.n, self.n), np.complex128, order="F")
        f = self.lib.oracle_compute_matrix_approx if approx else self.lib.oracle_compute_matrix
        f(self.s, float(freq), _p(Z))
        self.freq = float(freq)
        return Z

    def compute_matrix_cols(self, freq: float, c0: int, c1: int) -> np.ndarray:
        """Columns [c0, c1) of the quadrature-mode Z (a bounded sample for timing)."""
        Z = np.zeros((self.n, c1 - c0), np.complex128, order="F")
        self.lib.oracle_compute_matrix_cols(self.s, float(freq), int(c0), int(c1), _p(Z))
        return Z

    def compute_matrix_magnitudes(self, freq: float, c0: int = 0, c1: int | None = None) -> np.ndarray:
        """Columns [c0, c1) of M: M[j, i] = sum of the magnitudes of the terms that
        compute_matrix adds into Z[j, i] (quadrature mode). M / |Z| is the entry's
        cancellation factor; FP64 evaluations of Z[j, i] in different summation
        orders agree to a few ulps of M[j, i]."""
        c1 = self.n if c1 is None else c1
        M = np.zeros((self.n, c1 - c0), order="F")
        self.lib.oracle_compute_matrix_magnitudes(self.s, float(freq), int(c0), int(c1), _p(M))
        return M

    def reorient(self, tags, force: bool = False):
        t = np.asarray(tags, np.int32)
        signs = np.ones(self.n)
        r = self.lib.oracle_reorient(self.s, len(t), _p(t), int(force), _p(signs))
        if r < 0:
            raise ValueError("delta gap not connected")
        return signs if r == 1 else None

    def rhs_delta_gap(self, freq, tags, V0=1.0, signs=None) -> np.ndarray:
        V = np.zeros(self.n, np.complex128)
        t = np.asarray(tags, np.int32)
        s = None if signs is None else np.ascontiguousarray(signs, np.float64)
        self.lib.oracle_rhs_delta_gap(self.s, float(freq), len(t), _p(t), complex(V0).real, complex(V0).imag, _p(s),
                                      _p(V))
        return V

    def rhs_plane_wave(self, freq, theta, phi, Etheta=1.0, Ephi=1.0) -> np.ndarray:
        V = np.zeros(self.n, np.complex128)
        a, b = complex(Etheta), complex(Ephi)
        self.lib.oracle_rhs_plane_wave(self.s, float(freq), float(theta), float(phi), a.real, a.imag, b.real, b.imag,
                                       _p(V))
        return V

    @staticmethod
    def solve(Z: np.ndarray, V: np.ndarray, symmetric: bool = False) -> np.ndarray:
        """zgetrf+zgetrs (solve_general) or zsytrf+zsytrs (solve_symmetric)."""
        from scipy.linalg import lapack
        A = np.array(Z, np.complex128, order="F", copy=True)
        B = np.array(V, np.complex128, order="F", copy=True)
        if symmetric:
            ldu, ipiv, info = lapack.zsytrf(A, lower=0)
            if info != 0:
                raise np.linalg.LinAlgError(f"ZSYTRF info={info}")
            x, info = lapack.zsytrs(ldu, ipiv, B, lower=0)
        else:
            lu, piv, info = lapack.zgetrf(A, overwrite_a=1)
            if info != 0:
                raise np.linalg.LinAlgError(f"ZGETRF singular matrix (info={info})")
            x, info = lapack.zgetrs(lu, piv, B)
        if info != 0:
            raise np.linalg.LinAlgError("ZGETRS failed")
        return x

    def lump(self, freq, I):
        I = np.ascontiguousarray(I, np.complex128)
        AJ = np.zeros((self.nt, 3), np.complex128)
        AdivJ = np.zeros(self.nt, np.complex128)
        J = np.zeros((self.nt, 3), np.complex128)
        self.lib.oracle_lump(self.s, float(freq), _p(I), _p(AJ), _p(AdivJ), _p(J))
        self.freq = float(freq)
        return AJ, AdivJ, J

    def eval_fields(self, points):
        P = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        E = np.zeros((P.shape[0], 3), np.complex128)
        H = np.zeros((P.shape[0], 3), np.complex128)
        self.lib.oracle_eval_fields(self.s, P.shape[0], _p(P), _p(E), _p(H))
        return E, H

    def port_values(self, I, rwg_table, tags, V0=1.0, signs=None, Z0=50.0) -> dict:
        """compute_port_values, src/emw_ana_antenna.cpp:76-105."""
        cur, pw = 0j, 0j
        V0 = complex(V0)
        for i in range(self.n):
            if not rwg_table[i, 13]:
                continue
            for t in tags:
                if int(rwg_table[i, 14]) == t:
                    s = 1.0 if signs is None else signs[i]
                    Ii = rwg_table[i, 10] * I[i] * s
                    cur += Ii
                    pw += 0.5 * V0 * np.conj(Ii)
        Z = V0 / cur
        g = (Z - Z0) / (Z + Z0)
        return {"current": cur, "power": pw, "impedance": Z, "gamma": g,
                "swr": (1 + abs(g)) / (1 - abs(g))}

    def gain(self, pwr: float, R: float, plane: int) -> np.ndarray:
        """compute_gain, src/emw_ana_antenna.cpp:33-65."""
        th = np.arange(360) * np.pi / 180
        c, s = np.cos(th), np.sin(th)
        z = np.zeros(360)
        P = {0: np.stack([R * c, R * s, z], 1), 1: np.stack([z, R * c, R * s], 1),
             2: np.stack([-R * c, z, R * s], 1)}[plane]
        E, H = self.eval_fields(P)
        S = 0.5 * np.cross(E, np.conj(H))
        Prad = np.sqrt(np.sum(np.abs(S) ** 2, axis=1))
        Rn = np.linalg.norm(P, axis=1)
        return 4 * np.pi * Rn * Rn * Prad / pwr

    def rcs(self, R: float, theta, phi) -> np.ndarray:
        """bistatic_RCS_unit_Ei at sph2rect(R, theta, phi)."""
        theta = np.asarray(theta, float)
        phi = np.asarray(phi, float)
        P = np.stack([R * np.cos(phi) * np.sin(theta), R * np.sin(phi) * np.sin(theta), R * np.cos(theta)], 1)
        E, _ = self.eval_fields(P)
        th = np.stack([np.cos(theta) * np.cos(phi), np.cos(theta) * np.sin(phi), -np.sin(theta)], 1)
        ph = np.stack([-np.sin(phi), np.cos(phi), np.zeros_like(phi)], 1)
        Et = np.sum(th * E, axis=1)
        Ep = np.sum(ph * E, axis=1)
        return np.stack([4 * np.pi * R * R * np.abs(Et) ** 2, 4 * np.pi * R * R * np.abs(Ep) ** 2], 1)

    def bistatic_rcs(self, R: float = 10.0) -> np.ndarray:
        """The 359-angle loop of src/emw_ana_bistatic_rcs.cpp:102-117: rows {VV_t, HH_t, VV_p, HH_p}."""
        a = np.radians(np.arange(359.0))
        t = self.rcs(R, a, np.zeros(359))
        p = self.rcs(R, np.zeros(359), a)
        return np.concatenate([t, p], axis=1)
