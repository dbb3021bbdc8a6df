"""TEST INFRASTRUCTURE ONLY -- the oracle for the spherocylinder hot path.

Two CPU implementations of tmarschall/spherocyls' single-threaded src/cpp path,
behind the same Python surface:

* :class:`OracleBox` wraps ``liboracle.so``, a C restatement of the reference's
  algorithm (``spherocyl_oracle.c``; every routine cites the reference file:line
  it follows).  It is built by ``oracle/Makefile`` on any machine.
* :class:`RefBox` wraps ``_ref/libspherocyl_ref.so``, the reference's own sources
  compiled where they lie plus a small C-ABI shim (``ref_driver.cpp``).  It only
  exists where the reference checkout is present, and is used to pin the
  restatement and to produce the golden fixtures under ``tests/golden/``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this package, and only as the oracle the CUDA results are
compared with (or, in the benchmark, the timed CPU baseline).  The product library
(``spherocyls_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libspherocyl_ref.so")
# The reference checkout (its root, holding src/cpp and src/cuda) is named by the
# SPHEROCYLS_REF environment variable; without it nothing is built from it.
REF_ENV = "SPHEROCYLS_REF"


def ref_root() -> str | None:
    root = os.environ.get(REF_ENV)
    return root if root and os.path.isdir(root) else None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and, when $SPHEROCYLS_REF names the reference checkout,
    oracle/_ref from its src/cpp)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    root = ref_root()
    if with_ref is None:
        with_ref = root is not None and os.path.isdir(os.path.join(root, "src", "cpp"))
    if with_ref:
        if root is None:
            raise RuntimeError(f"{REF_ENV} does not name the reference checkout")
        subprocess.run(["make", "-s", "-C", HERE, "ref",
                        f"REF_SRC={os.path.join(root, 'src', 'cpp')}"], check=True)
        cuda = os.path.join(root, "src", "cuda")
        if os.path.isdir(cuda):
            subprocess.run(["make", "-s", "-C", HERE, "ref_cuda", f"REF_CUDA={cuda}"], check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def ref_available() -> bool:
    if not os.path.exists(REF_SO):
        return False
    try:
        ctypes.CDLL(REF_SO)
        return True
    except OSError:  # built for another architecture
        return False


class _Lib:
    """Binds one of the two libraries under a common prefix-free surface."""

    def __init__(self, path: str, prefix: str):
        self.lib = ctypes.CDLL(path)
        self.p = prefix
        L = self.lib
        handle = ctypes.c_void_p

        def fn(name, res, args):
            f = getattr(L, prefix + name)
            f.restype = res
            f.argtypes = args
            return f

        self.create = fn("create", handle, [ctypes.c_int, ctypes.c_double, _dp, _dp, _dp, _dp, _dp,
                                            ctypes.c_double])
        self.destroy = fn("destroy", None, [handle])
        self.find_neighbors = fn("find_neighbors", None, [handle])
        self.calc_forces = fn("calc_forces", None, [handle])
        self.calc_se = fn("calc_se", None, [handle])
        self.strain_step = fn("strain_step", None if prefix == "ref_" else ctypes.c_int, [handle])
        self.resize_step = fn("resize_step", None if prefix == "ref_" else ctypes.c_int,
                              [handle, ctypes.c_int])
        self.gd_step = fn("gd_step", None if prefix == "ref_" else ctypes.c_int, [handle])
        self.run_strain_steps = fn("run_strain_steps", ctypes.c_int, [handle, ctypes.c_int, _dp])
        self.run_resize_steps = fn("run_resize_steps", ctypes.c_int,
                                   [handle, ctypes.c_int, ctypes.c_int, _dp])
        self.run_gd_steps = fn("run_gd_steps", ctypes.c_int,
                               [handle, ctypes.c_int, ctypes.c_double, _dp])
        if prefix == "orc_":
            self.create_rect = fn("create_rect", handle,
                                  [ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp,
                                   _dp, _dp, ctypes.c_double])
            self.run_pure_steps = fn("run_pure_steps", ctypes.c_int, [handle, ctypes.c_int, _dp])
            self.cg_minimize = fn("cg_minimize", ctypes.c_int,
                                  [handle, ctypes.c_int, _ip, _dp, _ip])
            self.strain_to_gamma = fn("strain_to_gamma", ctypes.c_long, [handle, ctypes.c_double])
        self.n = fn("n", ctypes.c_int, [handle])
        self.get_state = fn("get_state", None, [handle, _dp, _dp, _dp])
        self.get_forces = fn("get_forces", None, [handle, _dp, _dp, _dp])
        self.get_moved = fn("get_moved", None, [handle, _dp, _dp])
        self.get_consts = fn("get_consts", None, [handle, _dp, _dp])
        self.get_scalars = fn("get_scalars", None, [handle, _dp])
        self.get_se = fn("get_se", None, [handle, _dp])
        self.get_pairs = fn("get_pairs", ctypes.c_long, [handle, _ip, ctypes.c_long])
        if prefix == "orc_":
            for name in ("set_strain_rate", "set_resize_rate", "set_step", "set_gamma",
                         "set_total_gamma"):
                setattr(self, name, fn(name, None, [handle, ctypes.c_double]))
            self.zero_pyx = fn("zero_pyx", None, [handle])
            self.set_two_point = fn("set_two_point", None, [handle, ctypes.c_int])
        else:
            self.set_params = fn("set_params", None, [handle] + [ctypes.c_double] * 5)


_LIBS: dict[str, _Lib] = {}


def _lib(kind: str) -> _Lib:
    if kind not in _LIBS:
        if kind == "orc":
            if not os.path.exists(ORACLE_SO):
                build(with_ref=False)
            _LIBS[kind] = _Lib(ORACLE_SO, "orc_")
        else:
            if not ref_available():
                raise RuntimeError("reference build oracle/_ref is not available on this machine")
            _LIBS[kind] = _Lib(REF_SO, "ref_")
    return _LIBS[kind]


def generate_packing(n: int, packing: float, a_over_r: float, r_small: float = 0.5,
                     r_ratio: float = 1.4, seed: int = 0, min_sep: float = 0.1):
    """The benchmark workload's seeded crossing-free packing (the library's
    generate_packing, restated so that the CPU arm needs no product code):
    returns (L, x, y, phi, R, A)."""
    L = _lib("orc").lib
    f = L.orc_generate_packing
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_uint64, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
    x, y, p, R, A = (np.empty(n) for _ in range(5))
    out = ctypes.c_double()
    rc = f(int(n), float(packing), float(a_over_r), float(r_small), float(r_ratio),
           ctypes.c_uint64(int(seed)), float(min_sep), _ptr(x), _ptr(y), _ptr(p), _ptr(R), _ptr(A),
           ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle packing generation failed ({rc})")
    return out.value, x, y, p, R, A


class _BoxBase:
    """One periodic square box of spherocylinders, in the reference's particle order."""

    kind = "orc"

    def __init__(self, L, x, y, phi, A, R, pad=0.0, *, strain_rate=0.0, resize_rate=0.0,
                 step=0.05, gamma=0.0, total_gamma=0.0, two_point=False, Ly=None):
        if two_point and self.kind != "orc":
            raise ValueError("the two-point contact rule exists only in the restatement")
        if Ly is not None and self.kind != "orc":
            raise ValueError("the reference's src/cpp box is square")
        self._L = _lib(self.kind)
        x, y, phi, A, R = (_f64(v) for v in (x, y, phi, A, R))
        self.n = int(x.shape[0])
        if Ly is None:
            self.h = self._L.create(self.n, float(L), _ptr(x), _ptr(y), _ptr(phi), _ptr(A),
                                    _ptr(R), float(pad))
        else:
            self.h = self._L.create_rect(self.n, float(L), float(Ly), _ptr(x), _ptr(y), _ptr(phi),
                                         _ptr(A), _ptr(R), float(pad))
        if not self.h:
            raise RuntimeError("oracle box creation failed")
        self.set_params(strain_rate=strain_rate, resize_rate=resize_rate, step=step, gamma=gamma,
                        total_gamma=total_gamma)
        if two_point:
            self._L.set_two_point(self.h, 1)
        # The reference's constructor leaves the forces uninitialised (new Spherocyl[n]);
        # its run methods always call calc_se/calc_forces before the first step
        # (src/cpp/strain_dynamics.cpp:242-279), so do the same here.
        self.calc_forces()

    def set_params(self, *, strain_rate, resize_rate, step, gamma, total_gamma):
        L = self._L
        if self.kind == "orc":
            L.set_strain_rate(self.h, strain_rate)
            L.set_resize_rate(self.h, resize_rate)
            L.set_step(self.h, step)
            L.set_gamma(self.h, gamma)
            L.set_total_gamma(self.h, total_gamma)
        else:
            L.set_params(self.h, strain_rate, resize_rate, step, gamma, total_gamma)

    def close(self):
        if getattr(self, "h", None):
            self._L.destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- per-step routines -------------------------------------------------
    def find_neighbors(self):
        self._L.find_neighbors(self.h)

    def calc_forces(self):
        self._L.calc_forces(self.h)

    def calc_se(self):
        self._L.calc_se(self.h)

    def strain_step(self):
        self._L.strain_step(self.h)

    def resize_step(self, shrink: bool):
        self._L.resize_step(self.h, int(bool(shrink)))

    def gd_step(self):
        self._L.gd_step(self.h)

    def run_strain_steps(self, nsteps: int, record_se: bool = False):
        out = np.zeros((nsteps, 5)) if record_se else None
        rc = self._L.run_strain_steps(self.h, int(nsteps), _ptr(out) if out is not None else None)
        if rc != 0:
            raise RuntimeError("oracle strain run failed")
        return out

    def run_resize_steps(self, nsteps: int, shrink: bool, record_se: bool = False):
        out = np.zeros((nsteps, 5)) if record_se else None
        rc = self._L.run_resize_steps(self.h, int(nsteps), int(bool(shrink)),
                                      _ptr(out) if out is not None else None)
        if rc != 0:
            raise RuntimeError("oracle resize run failed")
        return out

    def run_pure_steps(self, nsteps: int, record_se: bool = False):
        out = np.zeros((nsteps, 5)) if record_se else None
        rc = self._L.run_pure_steps(self.h, int(nsteps), _ptr(out) if out is not None else None)
        if rc != 0:
            raise RuntimeError("oracle pure-shear run failed")
        return out

    def strain_to_gamma(self, gamma_max: float) -> int:
        k = self._L.strain_to_gamma(self.h, float(gamma_max))
        if k < 0:
            raise RuntimeError("oracle strain_to_gamma failed")
        return k

    def cg_minimize(self, max_iter: int):
        """(iterations, energy, stop reason) of the conjugate-gradient restatement."""
        it = ctypes.c_int()
        e = ctypes.c_double()
        why = ctypes.c_int()
        if self._L.cg_minimize(self.h, int(max_iter), ctypes.byref(it), ctypes.byref(e),
                               ctypes.byref(why)) != 0:
            raise RuntimeError("oracle cg failed")
        return it.value, e.value, why.value

    def run_gd_steps(self, nsteps: int, emin: float = 0.0):
        out = np.zeros(nsteps)
        s = self._L.run_gd_steps(self.h, int(nsteps), float(emin), _ptr(out))
        return s, out[: min(s + 1, nsteps)]

    # --- state -------------------------------------------------------------
    def state(self):
        x, y, p = np.empty(self.n), np.empty(self.n), np.empty(self.n)
        self._L.get_state(self.h, _ptr(x), _ptr(y), _ptr(p))
        return x, y, p

    def forces(self):
        fx, fy, t = np.empty(self.n), np.empty(self.n), np.empty(self.n)
        self._L.get_forces(self.h, _ptr(fx), _ptr(fy), _ptr(t))
        return fx, fy, t

    def moved(self):
        xm, ym = np.empty(self.n), np.empty(self.n)
        self._L.get_moved(self.h, _ptr(xm), _ptr(ym))
        return xm, ym

    def consts(self):
        I, RC = np.empty(self.n), np.empty(self.n)
        self._L.get_consts(self.h, _ptr(I), _ptr(RC))
        return I, RC

    def scalars(self) -> dict:
        out = np.empty(10)
        self._L.get_scalars(self.h, _ptr(out))
        keys = ("Lx", "Ly", "gamma", "gamma_total", "pad", "W", "H", "packing", "rows", "cols")
        return dict(zip(keys, out.tolist()))

    def se(self) -> np.ndarray:
        """E, Pxx, Pyy, Pxy, Pyx as the reference accumulates them."""
        out = np.empty(5)
        self._L.get_se(self.h, _ptr(out))
        return out

    def pairs(self) -> np.ndarray:
        """Half neighbour list as an (M, 2) int array of (p, q), p < q, in list order."""
        m = self._L.get_pairs(self.h, None, 0)
        out = np.empty((max(m, 1), 2), dtype=np.int32)
        self._L.get_pairs(self.h, out.ctypes.data_as(_ip), m)
        return out[:m]


class OracleBox(_BoxBase):
    kind = "orc"


class RefBox(_BoxBase):
    kind = "ref"
