"""Python mirror of the reference's box object over the C ABI.

``SpherocylBox`` follows the interface of tmarschall/spherocyls' ``SpherocylBox``
(src/cpp/spherocyl_box.h:86-119): the constructor takes the box side, particle
arrays and the cell padding; setters for strain rate, resize rate, step, gamma and
total gamma; ``find_neighbors``, ``calc_forces``, ``calc_se``; the per-step
routines of ``run_strain`` / ``resize_box`` / ``gradient_descent_minimize``.  A
box may hold several independent systems that advance together (``BoxBatch``).
All work happens in libspherocyl on the GPU; this module only moves arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import PASS, PREC, STRESS, ScOptions, check, lib

_dp = ctypes.POINTER(ctypes.c_double)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def generate_packing(n: int, packing: float, a_over_r: float, r_small: float = 0.5,
                     r_ratio: float = 1.4, seed: int = 0, min_sep: float = 0.1):
    """Seeded crossing-free bidisperse packing: returns (L, x, y, phi, R, A)."""
    x, y, p, R, A = (np.empty(n) for _ in range(5))
    L = ctypes.c_double()
    st = lib().sc_generate_packing(int(n), float(packing), float(a_over_r), float(r_small),
                                   float(r_ratio), ctypes.c_uint64(int(seed)), float(min_sep),
                                   _ptr(x), _ptr(y), _ptr(p), _ptr(R), _ptr(A), ctypes.byref(L))
    if st != 0:
        raise _lib.ScError(st, "packing generation failed")
    return L.value, x, y, p, R, A


def generate_packing_device(n: int, packing: float, a_over_r: float, r_small: float = 0.5,
                            r_ratio: float = 1.4, seed: int = 0, min_sep: float = 0.1,
                            device: int = 0):
    """generate_packing's packing placed on the GPU (for large N): returns
    (L, x, y, phi, R, A); deterministic for a seed, a different sequence."""
    x, y, p, R, A = (np.empty(n) for _ in range(5))
    L = ctypes.c_double()
    st = lib().sc_generate_packing_device(int(device), int(n), float(packing), float(a_over_r),
                                          float(r_small), float(r_ratio),
                                          ctypes.c_uint64(int(seed)), float(min_sep), _ptr(x),
                                          _ptr(y), _ptr(p), _ptr(R), _ptr(A), ctypes.byref(L))
    if st != 0:
        raise _lib.ScError(st, "device packing generation failed")
    return L.value, x, y, p, R, A


def generate_config(n: int, packing: float, a_over_r: float, *, layout: str = "random",
                    angles: str = "random", angle_range=(0.0, 1.0), shear_angles: bool = False,
                    min_sep: float = 0.1, max_overlap: float = -1.0, a_sigma: float = 0.0,
                    r_small: float = 0.5, r_ratio: float = 1.4, seed: int = 0):
    """The reference's initial configurations (random / zero-energy / grid layouts;
    random, evenly spaced or aligned angles; Gamma-distributed a/R), seeded:
    returns (L, x, y, phi, R, A).  Zero energy: max_overlap=0.  Aligned:
    angle_range=(u, u)."""
    return _generate(n, packing, a_over_r, layout, angles, angle_range, shear_angles, min_sep,
                     max_overlap, a_sigma, r_small, r_ratio, seed, None)


def generate_config_rect(n: int, packing: float, a_over_r: float, box_aspect: float, *,
                         layout: str = "random", angles: str = "random", angle_range=(0.0, 1.0),
                         shear_angles: bool = False, min_sep: float = 0.1,
                         max_overlap: float = -1.0, a_sigma: float = 0.0, r_small: float = 0.5,
                         r_ratio: float = 1.4, seed: int = 0):
    """generate_config in a box of aspect Lx/Ly = box_aspect (the pure-shear start,
    src/cuda/main_pure_shear.cpp:168-170): returns (Lx, Ly, x, y, phi, R, A)."""
    return _generate(n, packing, a_over_r, layout, angles, angle_range, shear_angles, min_sep,
                     max_overlap, a_sigma, r_small, r_ratio, seed, float(box_aspect))


def _generate(n, packing, a_over_r, layout, angles, angle_range, shear_angles, min_sep,
              max_overlap, a_sigma, r_small, r_ratio, seed, box_aspect):
    from ._lib import ScGenOptions

    o = ScGenOptions()
    lib().sc_default_gen_options(ctypes.byref(o))
    o.layout = {"random": 0, "grid": 1}[layout]
    o.angle_mode = {"random": 0, "even": 1}[angles]
    o.angle_min, o.angle_max = float(angle_range[0]), float(angle_range[1])
    o.shear_angles = int(bool(shear_angles))
    o.min_sep, o.max_overlap, o.a_sigma = float(min_sep), float(max_overlap), float(a_sigma)
    x, y, p, R, A = (np.empty(n) for _ in range(5))
    L = ctypes.c_double()
    Ly = ctypes.c_double()
    if box_aspect is None:
        st = lib().sc_generate_config(ctypes.byref(o), int(n), float(packing), float(a_over_r),
                                      float(r_small), float(r_ratio), ctypes.c_uint64(int(seed)),
                                      _ptr(x), _ptr(y), _ptr(p), _ptr(R), _ptr(A),
                                      ctypes.byref(L))
    else:
        st = lib().sc_generate_config_rect(ctypes.byref(o), int(n), float(packing),
                                           float(a_over_r), float(r_small), float(r_ratio),
                                           box_aspect, ctypes.c_uint64(int(seed)), _ptr(x),
                                           _ptr(y), _ptr(p), _ptr(R), _ptr(A), ctypes.byref(L),
                                           ctypes.byref(Ly))
    if st != 0:
        raise _lib.ScError(st, "configuration generation failed")
    if box_aspect is None:
        return L.value, x, y, p, R, A
    return L.value, Ly.value, x, y, p, R, A


FMT = {"sp": 0, "sd": 1, "bin": 2}


def trim_memory(device: int = 0) -> None:
    """Return the device memory cached from destroyed handles to the driver."""
    check(lib().sc_trim_memory(int(device)), None)


def read_positions(path: str):
    """Read a position file (src/cpp or src/cuda text header, or the src/cuda binary
    layout for a path ending in .bin); returns (hdr, x, y, phi, R, A) with
    hdr = dict(Lx, Ly, packing, gamma, gamma_total, rate, dt)."""
    n = ctypes.c_int(0)
    hdr = np.empty(7)
    L = lib()
    st = L.sc_read_positions(path.encode(), ctypes.byref(n), _ptr(hdr), None, None, None, None,
                             None)
    check(st, None)
    x, y, p, R, A = (np.empty(n.value) for _ in range(5))
    st = L.sc_read_positions(path.encode(), ctypes.byref(n), _ptr(hdr), _ptr(x), _ptr(y), _ptr(p),
                             _ptr(R), _ptr(A))
    check(st, None)
    keys = ("Lx", "Ly", "packing", "gamma", "gamma_total", "rate", "dt")
    return dict(zip(keys, hdr.tolist())), x, y, p, R, A


def write_positions(path: str, hdr: dict, x, y, phi, R, A, fmt: str = "sd"):
    """Write a position file from host arrays (no GPU): hdr holds Lx, Ly, packing,
    gamma, gamma_total, rate, dt as read_positions returns them."""
    keys = ("Lx", "Ly", "packing", "gamma", "gamma_total", "rate", "dt")
    h = np.array([float(hdr[k]) for k in keys])
    x, y, phi, R, A = (_f64(v) for v in (x, y, phi, R, A))
    n = x.shape[0]
    if any(v.shape[0] != n for v in (y, phi, R, A)):
        raise ValueError("x, y, phi, R and A need the same length")
    check(lib().sc_write_positions(path.encode(), FMT[fmt], n, _ptr(h), _ptr(x), _ptr(y),
                                   _ptr(phi), _ptr(R), _ptr(A)), None)


class BoxBatch:
    """One or more independent periodic boxes advanced together on one GPU."""

    def __init__(self, n_per_sys, L, x, y, phi, A, R, pad=0.0, *, precision: str = "fp64",
                 stress: str = "compat", device: int = 0, max_nbrs: int = 0,
                 use_graphs: bool = True, block: int = 0, profile: bool = False,
                 contacts: int = 1, Ly=None, stage_inputs: bool = False,
                 cg_max_probes: int = 0, pass_kind: str = "auto", tile_target: int = 0,
                 persist_steps: bool = False):
        n_per_sys = np.ascontiguousarray(np.atleast_1d(n_per_sys), dtype=np.int32)
        self.nsys = int(n_per_sys.shape[0])
        self.n_per_sys = n_per_sys
        self.ntot = int(n_per_sys.sum())
        L = _f64(np.broadcast_to(np.asarray(L, dtype=np.float64), (self.nsys,)))
        pad = _f64(np.broadcast_to(np.asarray(pad, dtype=np.float64), (self.nsys,)))
        x, y, phi, A, R = (_f64(v) for v in (x, y, phi, A, R))
        for v in (x, y, phi, A, R):
            if v.shape[0] != self.ntot:
                raise ValueError("particle arrays must hold sum(n_per_sys) entries")
        opt = ScOptions()
        lib().sc_default_options(ctypes.byref(opt))
        opt.precision = PREC[precision]
        opt.stress_mode = STRESS[stress]
        opt.device = int(device)
        opt.max_nbrs = int(max_nbrs)
        opt.use_graphs = int(bool(use_graphs))
        opt.block = int(block)
        opt.profile = int(bool(profile))
        if int(contacts) not in (1, 2):
            raise ValueError("contacts must be 1 (one contact per pair) or 2")
        opt.contact_model = 1 if int(contacts) == 2 else 0
        opt.stage_inputs = int(bool(stage_inputs))
        opt.cg_max_probes = int(cg_max_probes)
        if pass_kind not in PASS:
            raise ValueError("pass_kind must be 'auto', 'list' or 'tile'")
        opt.pass_kind = PASS[pass_kind]
        opt.tile_target = int(tile_target)
        opt.persist_steps = int(bool(persist_steps))
        self.precision = precision
        h = ctypes.c_void_p()
        nps = n_per_sys.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        if Ly is None:
            st = lib().sc_create(ctypes.byref(opt), self.nsys, nps, _ptr(L), _ptr(pad), _ptr(x),
                                 _ptr(y), _ptr(phi), _ptr(R), _ptr(A), ctypes.byref(h))
        else:
            # rectangular boxes Lx = L, Ly (the src/cuda box)
            Ly = _f64(np.broadcast_to(np.asarray(Ly, dtype=np.float64), (self.nsys,)))
            st = lib().sc_create_rect(ctypes.byref(opt), self.nsys, nps, _ptr(L), _ptr(Ly),
                                      _ptr(pad), _ptr(x), _ptr(y), _ptr(phi), _ptr(R), _ptr(A),
                                      ctypes.byref(h))
        check(st, None)
        self.h = h

    # --- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            lib().sc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st):
        check(st, self.h)

    # --- setters (spherocyl_box.h:112-119) ----------------------------------
    def set_strain_rate(self, v, sys=-1):
        self._chk(lib().sc_set_strain_rate(self.h, sys, float(v)))

    def set_resize_rate(self, v, sys=-1):
        self._chk(lib().sc_set_resize_rate(self.h, sys, float(v)))

    def set_step(self, v, sys=-1):
        self._chk(lib().sc_set_step(self.h, sys, float(v)))

    def set_gamma(self, v, sys=-1):
        self._chk(lib().sc_set_gamma(self.h, sys, float(v)))

    def set_total_gamma(self, v, sys=-1):
        self._chk(lib().sc_set_total_gamma(self.h, sys, float(v)))

    def set_stream(self, stream_ptr: int | None):
        self._chk(lib().sc_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        self._chk(lib().sc_synchronize(self.h))

    # --- compute ----------------------------------------------------------
    def find_neighbors(self):
        self._chk(lib().sc_find_neighbors(self.h))

    def calc_forces(self):
        self._chk(lib().sc_calc_forces(self.h))

    def calc_se(self) -> np.ndarray:
        """(nsys, 5): E, Pxx, Pyy, Pxy, Pyx per system."""
        out = np.empty((self.nsys, 5))
        self._chk(lib().sc_calc_se(self.h, _ptr(out)))
        return out

    def strain_steps(self, nsteps: int, se_every: int = 0):
        out = None
        if se_every > 0 and nsteps // se_every > 0:
            out = np.empty((nsteps // se_every, self.nsys, 5))
        self._chk(lib().sc_strain_steps(self.h, int(nsteps), int(se_every),
                                        _ptr(out) if out is not None else None))
        return out

    def resize_steps(self, nsteps: int, shrink: bool = True, se_every: int = 0):
        out = None
        if se_every > 0 and nsteps // se_every > 0:
            out = np.empty((nsteps // se_every, self.nsys, 5))
        self._chk(lib().sc_resize_steps(self.h, int(nsteps), int(bool(shrink)), int(se_every),
                                        _ptr(out) if out is not None else None))
        return out

    def strain_to_gamma(self, gamma_max: float) -> int:
        """Shear without setting gamma back until gamma >= gamma_max (run_strain
        (dGammaMax), src/cuda/strain_dynamics.cu:1097-1108); returns the steps."""
        k = ctypes.c_long()
        self._chk(lib().sc_strain_to_gamma(self.h, float(gamma_max), ctypes.byref(k)))
        return k.value

    def pure_strain_steps(self, nsteps: int, se_every: int = 0):
        """Pure shear at each system's strain rate (pure_strain_step_2p,
        src/cuda/2point_dynamics.cu:2180-2283): x stretched, y compressed."""
        out = None
        if se_every > 0 and nsteps // se_every > 0:
            out = np.empty((nsteps // se_every, self.nsys, 5))
        self._chk(lib().sc_pure_strain_steps(self.h, int(nsteps), int(se_every),
                                             _ptr(out) if out is not None else None))
        return out

    def gd_minimize(self, max_steps: int, e_min: float = 0.0):
        steps = ctypes.c_int()
        ef = ctypes.c_double()
        self._chk(lib().sc_gd_minimize(self.h, int(max_steps), float(e_min), ctypes.byref(steps),
                                       ctypes.byref(ef)))
        return steps.value, ef.value

    # --- minimisation and quasistatic compression -------------------------------
    def cg_minimize(self, max_iter: int = 100000):
        """The reference's Polak-Ribiere conjugate gradient (cjpr_relax_2p,
        src/cuda/2point_dynamics.cu:4233-4296) on every system: returns per-system
        (iterations, energy, stop reason) with reason 1 zero force, 2 three equal
        energies, 3 no lower energy along any direction, 4 max_iter, 5 a line search
        that reached the probe cap (the handle's cg_max_probes)."""
        it = np.zeros(self.nsys, dtype=np.int32)
        e = np.zeros(self.nsys)
        why = np.zeros(self.nsys, dtype=np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        st = lib().sc_cg_minimize(self.h, int(max_iter), it.ctypes.data_as(ip), _ptr(e),
                                  why.ctypes.data_as(ip))
        if st not in (0, _lib.SC_E_NOCONV):
            self._chk(st)
        return it, e, why

    def fire_minimize(self, ftol: float, max_iter: int = 100000, dt0: float = 1e-2,
                      dt_max: float = 0.2):
        """FIRE until max|F| < ftol per system; returns (iters, fmax[nsys], done[nsys])."""
        it = ctypes.c_int()
        fm = np.empty(self.nsys)
        dn = np.empty(self.nsys, dtype=np.int32)
        st = lib().sc_fire_minimize(self.h, float(ftol), int(max_iter), float(dt0), float(dt_max),
                                    ctypes.byref(it), _ptr(fm),
                                    dn.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if st not in (0, _lib.SC_E_NOCONV):
            self._chk(st)
        return it.value, fm, dn.astype(bool)

    def fire_iterations(self) -> np.ndarray:
        """Per-system iterations of the last fire_minimize."""
        it = np.zeros(self.nsys, dtype=np.int32)
        self._chk(lib().sc_fire_iterations(self.h, it.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return it

    def rotate_shear(self, sys: int = -1):
        """Turn to the frame in which the sheared cell is upright (rotate_by_gamma)."""
        self._chk(lib().sc_rotate_shear(self.h, int(sys)))

    def flip_shear(self, sys: int = -1):
        """Reverse the shear direction (x -> Lx - x, phi -> -phi, gamma -> -gamma)."""
        self._chk(lib().sc_flip_shear(self.h, int(sys)))

    def affine_scale(self, factor: float, sys: int = -1):
        self._chk(lib().sc_affine_scale(self.h, int(sys), float(factor)))

    def quasistatic_compress(self, dphi: float, ftol: float, e_jam: float,
                             max_increments: int = 100000, max_iter: int = 100000):
        """Affine steps of dphi + FIRE until E/N > e_jam; returns (phi_jam[nsys], n_inc)."""
        pj = np.empty(self.nsys)
        n = ctypes.c_int()
        self._chk(lib().sc_quasistatic_compress(self.h, float(dphi), float(ftol), float(e_jam),
                                                int(max_increments), int(max_iter), _ptr(pj),
                                                ctypes.byref(n)))
        return pj, n.value

    def autotune(self, steps: int = 50):
        """Pick the neighbour-list padding, the force pass (per particle or by tiles)
        and its block or tile size of the mixed form by timing copies of this batch;
        returns (pad_factor, block) -- the pass and tile size are in options()."""
        f = ctypes.c_double()
        b = ctypes.c_int()
        self._chk(lib().sc_autotune(self.h, int(steps), ctypes.byref(f), ctypes.byref(b)))
        return f.value, b.value

    def options(self) -> dict:
        """The handle's current options (pass kind, block, tile size, ...)."""
        o = ScOptions()
        self._chk(lib().sc_get_options(self.h, ctypes.byref(o)))
        kinds = {v: k for k, v in PASS.items()}
        return {"precision": o.precision, "block": o.block, "contact_model": o.contact_model,
                "pass_kind": kinds.get(o.pass_kind, o.pass_kind), "tile_target": o.tile_target,
                "cg_max_probes": o.cg_max_probes, "persist_steps": bool(o.persist_steps)}

    def find_jam(self, e_jam: float, step: float = 1e-3, min_step: float = 1e-12,
                 ftol: float = 1e-13, max_iter: int = 200000, max_steps: int = 10000):
        """Bisect each system's packing fraction to energy per particle e_jam
        (find_jam_2p); returns (phi[nsys], resizes made), phi negated where
        max_steps ran out first.  Raises ScError (SC_E_NOCONV) if a phase's step
        grows to 1 before the energy crosses e_jam."""
        pj = np.empty(self.nsys)
        n = ctypes.c_int()
        self._chk(lib().sc_find_jam(self.h, float(e_jam), float(step), float(min_step),
                                    float(ftol), int(max_iter), int(max_steps), _ptr(pj),
                                    ctypes.byref(n)))
        return pj, n.value

    # --- runs with file output (single-system handles) -------------------------
    def save_positions(self, path: str, fmt: str = "sp", sys: int = 0):
        self._chk(lib().sc_save_positions(self.h, int(sys), path.encode(), FMT[fmt]))

    def run_strain(self, out_dir: str, run_gamma: float, pos_save: float, se_save: float,
                   t_start: int = 0, fmt: str = "sp") -> int:
        t = ctypes.c_ulong()
        self._chk(lib().sc_run_strain(self.h, out_dir.encode(), float(run_gamma), float(pos_save),
                                      float(se_save), int(t_start), FMT[fmt], ctypes.byref(t)))
        return t.value

    def run_resize(self, out_dir: str, final_packing: float, pos_save: float, se_save: float,
                   t_start: int = 0, fmt: str = "sp") -> int:
        t = ctypes.c_ulong()
        self._chk(lib().sc_run_resize(self.h, out_dir.encode(), float(final_packing),
                                      float(pos_save), float(se_save), int(t_start), FMT[fmt],
                                      ctypes.byref(t)))
        return t.value

    def run_pure_strain(self, out_dir: str, stop_aspect: float, pos_save: float, se_save: float,
                        t_start: int = 0, fmt: str = "sd") -> int:
        t = ctypes.c_ulong()
        self._chk(lib().sc_run_pure_strain(self.h, out_dir.encode(), float(stop_aspect),
                                           float(pos_save), float(se_save), int(t_start),
                                           FMT[fmt], ctypes.byref(t)))
        return t.value

    def run_minimize(self, out_dir: str, max_steps: int, e_min: float = 0.0,
                     pos_save_n: int = 1000) -> int:
        s = ctypes.c_int()
        self._chk(lib().sc_run_minimize(self.h, out_dir.encode(), int(max_steps), float(e_min),
                                        int(pos_save_n), ctypes.byref(s)))
        return s.value

    def run_find_jam(self, out_dir: str, e_jam: float, step: float, ftol: float = 1e-13,
                     max_iter: int = 200000):
        """find_jam_2p with its files; e_jam per unit area as there.  Returns
        (packing fraction, resizes made)."""
        s = ctypes.c_int()
        phi = ctypes.c_double()
        self._chk(lib().sc_run_find_jam(self.h, out_dir.encode(), float(e_jam), float(step),
                                        float(ftol), int(max_iter), ctypes.byref(s),
                                        ctypes.byref(phi)))
        return phi.value, s.value

    def run_y_compress(self, out_dir: str, e_target: float, step: float, ftol: float = 1e-13,
                       max_iter: int = 200000):
        """y_compress_energy_2p with its files: find_jam_2p's bisection resizing Ly
        and y alone.  Returns (packing fraction, resizes made)."""
        s = ctypes.c_int()
        phi = ctypes.c_double()
        self._chk(lib().sc_run_y_compress(self.h, out_dir.encode(), float(e_target), float(step),
                                          float(ftol), int(max_iter), ctypes.byref(s),
                                          ctypes.byref(phi)))
        return phi.value, s.value

    def run_qs_compress(self, out_dir: str, final_packing: float, step: float,
                        ftol: float = 1e-13, max_iter: int = 1000000) -> int:
        """compress_qs2p (expand_qs2p below the current packing fraction) with its
        files; returns the resizes made."""
        s = ctypes.c_int()
        self._chk(lib().sc_run_qs_compress(self.h, out_dir.encode(), float(final_packing),
                                           float(step), float(ftol), int(max_iter),
                                           ctypes.byref(s)))
        return s.value

    # --- state ------------------------------------------------------------
    def state(self, out=None):
        """(x, y, phi) in input order; `out`: three caller arrays of ntot float64 (for
        example in pinned host memory) to read into instead of new ones."""
        if out is None:
            x, y, p = (np.empty(self.ntot) for _ in range(3))
        else:
            x, y, p = out
            for a in (x, y, p):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and
                        a.flags.c_contiguous and a.size == self.ntot):
                    raise ValueError("state(out=...): three contiguous float64 arrays of ntot")
        self._chk(lib().sc_get_state(self.h, _ptr(x), _ptr(y), _ptr(p)))
        return x, y, p

    def forces(self):
        fx, fy, t = (np.empty(self.ntot) for _ in range(3))
        self._chk(lib().sc_get_forces(self.h, _ptr(fx), _ptr(fy), _ptr(t)))
        return fx, fy, t

    def box(self, sys: int = 0) -> dict:
        out = np.empty(10)
        self._chk(lib().sc_get_box(self.h, int(sys), _ptr(out)))
        keys = ("Lx", "Ly", "gamma", "gamma_total", "pad", "W", "H", "packing", "rows", "cols")
        return dict(zip(keys, out.tolist()))

    def pairs(self, sys: int = 0) -> np.ndarray:
        n = ctypes.c_long()
        self._chk(lib().sc_get_pairs(self.h, int(sys), None, 0, ctypes.byref(n)))
        out = np.empty((max(n.value, 1), 2), dtype=np.int32)
        self._chk(lib().sc_get_pairs(self.h, int(sys), out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int)), n.value, ctypes.byref(n)))
        return out[: n.value]

    def counters(self) -> dict:
        out = (ctypes.c_longlong * 4)()
        self._chk(lib().sc_get_counters(self.h, out))
        return {"steps": out[0], "rebuilds": out[1], "status": out[2], "kernels": out[3]}

    def pass_times(self) -> dict:
        out = np.empty(6)
        self._chk(lib().sc_get_pass_times(self.h, _ptr(out)))
        return {"corr_ms": out[0], "pred_ms": out[1], "rebuild_ms": out[2],
                "n_corr": int(out[3]), "n_pred": int(out[4]), "n_rebuild": int(out[5])}


class SpherocylBox(BoxBatch):
    """A single periodic square box: SpherocylBox(L, N, x, y, phi, A*, R*, pad)."""

    def __init__(self, L, x, y, phi, A, R, pad=0.0, **kw):
        x = _f64(x)
        super().__init__([x.shape[0]], [L], x, y, phi, A, R, [pad], **kw)

    def calc_se(self) -> np.ndarray:
        return super().calc_se()[0]
