"""FRICO's own sources, compiled in place (oracle/_ref/libfrico_ref.so) -- TEST INFRASTRUCTURE.

Available only on a machine with the FRICO checkout (see oracle/ref/Makefile);
used to pin the oracle restatement and to generate tests/golden/ fixtures.
Single global simulation inside the library: one RefFrico at a time.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libfrico_ref.so"
_lib = None


def available() -> bool:
    return LIB.exists()


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(LIB))
        vp, l, i, d = C.c_void_p, C.c_long, C.c_int, C.c_double
        sig = {
            "ref_load": ([l, vp, l, vp, vp, l, vp, vp, i, i, i], l),
            "ref_num_tri": ([], l),
            "ref_get_rwg": ([vp], None),
            "ref_dunavant": ([i, vp, vp, vp, vp], i),
            "ref_integrate_subtri": ([l, i, vp], i),
            "ref_compute_matrix": ([d, i, vp], None),
            "ref_reorient": ([i, vp, i, vp], i),
            "ref_update_rhs_delta_gap": ([d, i, vp, d, d, vp], None),
            "ref_update_rhs_plane_wave": ([d, d, d, d, d, d, d, vp], None),
            "ref_run_context_delta_gap": ([d, i, vp, d, d, vp, vp, vp, vp], i),
            "ref_run_context_plane_wave": ([d, d, d, d, d, d, d, vp, vp, vp, vp], i),
            "ref_eval_fields": ([l, vp, vp, vp], None),
            "ref_port_values": ([i, vp, d, d, d, vp], None),
            "ref_gain": ([d, d, i, vp], None),
            "ref_bistatic": ([d, vp], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def dunavant(degree, p0, p1, p2):
    lib = _load()
    out = np.zeros((100, 4))
    a, b, c = (np.ascontiguousarray(x, np.float64) for x in (p0, p1, p2))
    k = lib.ref_dunavant(degree, _p(a), _p(b), _p(c), _p(out))
    return out[:k].copy()


class RefFrico:
    def __init__(self, mesh, degree: int = 1, approx: bool = False, force_symmetry: bool = False):
        self.lib = _load()
        V = np.ascontiguousarray(mesh.vertices, np.float64)
        T = np.ascontiguousarray(mesh.triangles, np.int64)
        tg = np.ascontiguousarray(mesh.tri_tags, np.int32)
        Cv = np.ascontiguousarray(mesh.curves, np.int64).reshape(-1, 2)
        Ct = np.ascontiguousarray(mesh.curve_tags, np.int32)
        n = self.lib.ref_load(V.shape[0], _p(V), T.shape[0], _p(T), _p(tg), Cv.shape[0], _p(Cv), _p(Ct), degree,
                              int(approx), int(force_symmetry))
        if n < 0:
            raise ValueError({-1: "multiple_triangles", -2: "lonely_edge"}[n])
        self.n = int(n)
        self.nt = int(self.lib.ref_num_tri())

    def rwg(self):
        out = np.zeros((self.n, 17))
        self.lib.ref_get_rwg(_p(out))
        return out

    def integrate_subtri(self, t, degree):
        out = np.zeros((300, 4))
        k = self.lib.ref_integrate_subtri(int(t), degree, _p(out))
        return out[:k].copy()

    def compute_matrix(self, freq, approx=False):
        Z = np.zeros((self.n, self.n), np.complex128, order="F")
        self.lib.ref_compute_matrix(float(freq), int(approx), _p(Z))
        return Z

    def reorient(self, tags, force=False):
        t = np.asarray(tags, np.int32)
        s = np.zeros(self.n)
        r = self.lib.ref_reorient(len(t), _p(t), int(force), _p(s))
        return s if r else None

    def rhs_delta_gap(self, freq, tags, V0=1.0):
        t = np.asarray(tags, np.int32)
        V = np.zeros(self.n, np.complex128)
        v = complex(V0)
        self.lib.ref_update_rhs_delta_gap(float(freq), len(t), _p(t), v.real, v.imag, _p(V))
        return V

    def rhs_plane_wave(self, freq, theta, phi, Etheta=1.0, Ephi=1.0):
        V = np.zeros(self.n, np.complex128)
        a, b = complex(Etheta), complex(Ephi)
        self.lib.ref_update_rhs_plane_wave(float(freq), float(theta), float(phi), a.real, a.imag, b.real, b.imag,
                                           _p(V))
        return V

    def _outs(self):
        return (np.zeros(self.n, np.complex128), np.zeros((self.nt, 3), np.complex128),
                np.zeros(self.nt, np.complex128), np.zeros((self.nt, 3), np.complex128))

    def run_context_delta_gap(self, freq, tags, V0=1.0):
        I, AJ, AD, J = self._outs()
        t = np.asarray(tags, np.int32)
        v = complex(V0)
        rc = self.lib.ref_run_context_delta_gap(float(freq), len(t), _p(t), v.real, v.imag, _p(I), _p(AJ), _p(AD),
                                                _p(J))
        if rc != 0:
            raise np.linalg.LinAlgError("FRICO solve failed")
        return I, AJ, AD, J

    def run_context_plane_wave(self, freq, theta, phi, Etheta=1.0, Ephi=1.0):
        I, AJ, AD, J = self._outs()
        a, b = complex(Etheta), complex(Ephi)
        rc = self.lib.ref_run_context_plane_wave(float(freq), float(theta), float(phi), a.real, a.imag, b.real,
                                                 b.imag, _p(I), _p(AJ), _p(AD), _p(J))
        if rc != 0:
            raise np.linalg.LinAlgError("FRICO solve failed")
        return I, AJ, AD, J

    def eval_fields(self, points):
        P = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        E = np.zeros((P.shape[0], 3), np.complex128)
        H = np.zeros((P.shape[0], 3), np.complex128)
        self.lib.ref_eval_fields(P.shape[0], _p(P), _p(E), _p(H))
        return E, H

    def port_values(self, tags, V0=1.0, Z0=50.0):
        t = np.asarray(tags, np.int32)
        out = np.zeros(9)
        v = complex(V0)
        self.lib.ref_port_values(len(t), _p(t), v.real, v.imag, float(Z0), _p(out))
        return {"current": complex(out[0], out[1]), "power": complex(out[2], out[3]),
                "impedance": complex(out[4], out[5]), "gamma": complex(out[6], out[7]), "swr": out[8]}

    def gain(self, pwr, R, plane):
        out = np.zeros(360)
        self.lib.ref_gain(float(pwr), float(R), int(plane), _p(out))
        return out

    def bistatic_rcs(self, R=10.0):
        out = np.zeros((359, 4))
        self.lib.ref_bistatic(float(R), _p(out))
        return out
