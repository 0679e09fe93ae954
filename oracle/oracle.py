"""numpy front end of the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline, as the checker or the timed CPU baseline. Never part of the product path.

    Restatement   oracle/_build/liboracle.so  (oracle/bh_oracle.cpp): the reference's algorithms
                  restated in C++, FP64, with literal and intended multipole semantics.
    RefLiteral    oracle/_ref/libbhref.so: the reference's own compiled code (only where the
                  reference checkout was available at build time).
    RefScene      oracle/_ref/libbhref_solar.so: the reference's own scene set-up and ephemeris
                  parser (same condition).
All positions are (n, 3) float64; masses (n,) float64.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATEMENT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libbhref.so")
REF_SCENE_LIB = os.path.join(HERE, "_ref", "libbhref_solar.so")

P, S, D, I, L = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int, ctypes.c_long


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f64(a, cols=None):
    a = np.ascontiguousarray(a, np.float64)
    if cols is not None:
        assert a.ndim == 2 and a.shape[1] == cols
    return a


class Restatement:
    def __init__(self, path=RESTATEMENT_LIB):
        if not os.path.exists(path):
            raise RuntimeError(f"oracle not built: {path}")
        lib = ctypes.CDLL(path)
        lib.orc_bounds.argtypes = [P, S, P, P]
        lib.orc_morton_keys.argtypes = [P, S, D, P]
        lib.orc_sort_perm.argtypes = [P, S, P]
        lib.orc_tree_keys.argtypes = [P, S, P, D, P]
        lib.orc_guard.argtypes = [P, S, P, D]
        lib.orc_guard.restype = L
        lib.orc_build.argtypes = [P, P, S, P, D, I, I, S, P, P, P, P, P, P]
        lib.orc_build.restype = L
        lib.orc_force.argtypes = [P, P, S, P, D, I, I, D, D, P, S, I, P, P, P]
        lib.orc_direct.argtypes = [P, P, S, P, S, D, I, P, P]
        lib.orc_kick_drift.argtypes = [P, P, P, S, D]
        lib.orc_kick.argtypes = [P, P, S, D]
        lib.orc_steps.argtypes = [P, P, P, P, S, D, D, D, D, I, I, I, I, I, P, P]
        lib.orc_time_sample.argtypes = [P, P, S, P, D, I, I, D, D, P, S, I, P, P, P]
        lib.orc_frozen_record.argtypes = [P, P, P, S, D, D, D, D, I, I, I, P, P]
        lib.orc_frozen_record.restype = P
        lib.orc_frozen_run.argtypes = [P, P, P, P, I, P, P]
        lib.orc_frozen_entries.argtypes = [P]
        lib.orc_frozen_entries.restype = L
        lib.orc_frozen_free.argtypes = [P]
        lib.orc_direct_adjoint.argtypes = [P, P, P, S, D, D, I, P, P, I, P, P, P, P, P]
        lib.orc_solar_system.argtypes = [ctypes.c_uint64, S, P]
        lib.orc_decode_morton.argtypes = [P, S, D, P]
        self.lib = lib

    def decode_morton(self, keys, size):
        keys = np.ascontiguousarray(keys, np.uint64)
        out = np.zeros((len(keys), 3))
        self.lib.orc_decode_morton(_p(keys), len(keys), size, _p(out))
        return out

    def solar_system(self, seed, n):
        """The reference app's scene (SetupSolarSystem) with the library's draws: (n, 7) float64
        rows x, y, z, vx, vy, vz, m in SI units."""
        out = np.zeros((n, 7))
        self.lib.orc_solar_system(seed, n, _p(out))
        return out

    def bounds(self, pos):
        pos = _f64(pos, 3)
        c = np.zeros(3)
        s = np.zeros(1)
        self.lib.orc_bounds(_p(pos), len(pos), _p(c), _p(s))
        return c, float(s[0])

    def morton_keys(self, pos, size):
        pos = _f64(pos, 3)
        k = np.zeros(len(pos), np.uint64)
        self.lib.orc_morton_keys(_p(pos), len(pos), size, _p(k))
        return k

    def sort_perm(self, keys):
        keys = np.ascontiguousarray(keys, np.uint64)
        perm = np.zeros(len(keys), np.uint32)
        self.lib.orc_sort_perm(_p(keys), len(keys), _p(perm))
        return perm

    def tree_keys(self, pos, center, edge):
        pos = _f64(pos, 3)
        c = _f64(center)
        k = np.zeros(len(pos), np.uint64)
        self.lib.orc_tree_keys(_p(pos), len(pos), _p(c), edge, _p(k))
        return k

    def guard(self, pos, center, edge):
        pos = _f64(pos, 3)
        c = _f64(center)
        return int(self.lib.orc_guard(_p(pos), len(pos), _p(c), edge))

    def build(self, pos, mass, center, edge, leaf_capacity=1, mode=1):
        pos = _f64(pos, 3)
        mass = _f64(mass)
        c = _f64(center)
        n = len(pos)
        cap = 22 * n + 8
        keys = np.zeros(cap, np.uint64)
        counts = np.zeros(cap, np.int64)
        m = np.zeros(cap)
        com = np.zeros((cap, 3))
        cb = np.zeros(cap, np.uint8)
        q = np.zeros((cap, 6))
        got = self.lib.orc_build(_p(pos), _p(mass), n, _p(c), edge, leaf_capacity, mode, cap, _p(keys), _p(counts),
                                 _p(m), _p(com), _p(cb), _p(q))
        assert got >= 0
        return dict(keys=keys[:got], counts=counts[:got], mass=m[:got], com=com[:got], child_byte=cb[:got],
                    quad=q[:got])

    def force(self, pos, mass, center, edge, leaf_capacity, mode, theta, eps, targets=None, nthreads=1):
        pos = _f64(pos, 3)
        mass = _f64(mass)
        c = _f64(center)
        t = None if targets is None else np.ascontiguousarray(targets, np.uint32)
        nt = len(pos) if t is None else len(t)
        acc = np.zeros((nt, 3))
        nc = np.zeros(nt, np.int64)
        npp = np.zeros(nt, np.int64)
        self.lib.orc_force(_p(pos), _p(mass), len(pos), _p(c), edge, leaf_capacity, mode, theta, eps, _p(t),
                           0 if t is None else len(t), nthreads, _p(acc), _p(nc), _p(npp))
        return acc, nc, npp

    def direct(self, pos, mass, eps, targets=None, nthreads=1, potential=False):
        pos = _f64(pos, 3)
        mass = _f64(mass)
        t = None if targets is None else np.ascontiguousarray(targets, np.uint32)
        nt = len(pos) if t is None else len(t)
        acc = np.zeros((nt, 3))
        pot = np.zeros(nt)
        self.lib.orc_direct(_p(pos), _p(mass), len(pos), _p(t), nt, eps, nthreads, _p(acc), _p(pot))
        return (acc, pot) if potential else acc

    def steps(self, pos, vel, mass, acc, dt, theta, eps, edge_factor, leaf_capacity, mode, nsteps,
              acc_follows_body=1, nthreads=1):
        pos = _f64(pos, 3).copy()
        vel = _f64(vel, 3).copy()
        mass = _f64(mass).copy()
        acc = _f64(acc, 3).copy()
        perm = np.zeros(len(pos), np.uint32)
        stage = np.zeros(6)
        self.lib.orc_steps(_p(pos), _p(vel), _p(mass), _p(acc), len(pos), dt, theta, eps, edge_factor,
                           leaf_capacity, mode, nsteps, acc_follows_body, nthreads, _p(stage), _p(perm))
        return dict(pos=pos, vel=vel, mass=mass, acc=acc, perm=perm, stage_s=stage)

    def time_sample(self, pos, mass, center, edge, leaf_capacity, mode, theta, eps, targets, nthreads=1):
        pos = _f64(pos, 3)
        mass = _f64(mass)
        c = _f64(center)
        t = np.ascontiguousarray(targets, np.uint32)
        b = np.zeros(1)
        w = np.zeros(1)
        acc = np.zeros((len(t), 3))
        self.lib.orc_time_sample(_p(pos), _p(mass), len(pos), _p(c), edge, leaf_capacity, mode, theta, eps, _p(t),
                                 len(t), nthreads, _p(b), _p(w), _p(acc))
        return float(b[0]), float(w[0]), acc


class FrozenTrajectory:
    """FP64 KDK trajectory of the library's differentiable path with the interaction lists of
    its own forward pass held fixed; run() re-evaluates that map from another initial state
    (the function whose finite differences the adjoint must match)."""

    def __init__(self, orc, pos, vel, mass, dt, theta, eps, edge_factor, leaf_capacity, nsteps, nthreads=8):
        self.lib = orc.lib
        self.n = len(pos)
        self.nthreads = nthreads
        pos, vel, mass = _f64(pos, 3), _f64(vel, 3), _f64(mass)
        self.final_pos = np.zeros_like(pos)
        self.final_vel = np.zeros_like(vel)
        self.h = self.lib.orc_frozen_record(_p(pos), _p(vel), _p(mass), self.n, dt, theta, eps, edge_factor,
                                            leaf_capacity, nsteps, nthreads, _p(self.final_pos), _p(self.final_vel))

    def entries(self):
        return self.lib.orc_frozen_entries(self.h)

    def run(self, pos, vel, mass):
        pos, vel, mass = _f64(pos, 3), _f64(vel, 3), _f64(mass)
        xo = np.zeros_like(pos)
        vo = np.zeros_like(vel)
        self.lib.orc_frozen_run(self.h, _p(pos), _p(vel), _p(mass), self.nthreads, _p(xo), _p(vo))
        return xo, vo

    def close(self):
        if self.h:
            self.lib.orc_frozen_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def direct_adjoint(orc, pos, vel, mass, dt, eps, nsteps, dl_dx, dl_dv=None, nthreads=8):
    """FP64 direct-sum KDK trajectory and its adjoint: (final pos, final vel, d pos0, d vel0, d mass)."""
    pos, vel, mass = _f64(pos, 3), _f64(vel, 3), _f64(mass)
    n = len(pos)
    gx = None if dl_dx is None else _f64(dl_dx, 3)
    gvin = None if dl_dv is None else _f64(dl_dv, 3)
    xo, vo = np.zeros((n, 3)), np.zeros((n, 3))
    gx0, gv0, gm = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
    orc.lib.orc_direct_adjoint(_p(pos), _p(vel), _p(mass), n, dt, eps, nsteps, _p(gx), _p(gvin), nthreads, _p(xo),
                               _p(vo), _p(gx0), _p(gv0), _p(gm))
    return xo, vo, gx0, gv0, gm


class RefLiteral:
    """The reference's own compiled hot path (REF-LITERAL)."""

    def __init__(self, path=REF_LIB):
        if not os.path.exists(path):
            raise RuntimeError(f"REF-LITERAL not built: {path}")
        lib = ctypes.CDLL(path)
        lib.ref_bounds.argtypes = [P, S, P, P]
        lib.ref_morton_keys.argtypes = [P, S, D, P]
        lib.ref_sort_bodies.argtypes = [P, S, P]
        lib.ref_guard.argtypes = [P, S, P, D]
        lib.ref_guard.restype = L
        lib.ref_build_nodes.argtypes = [P, P, S, P, D, S, P, P, P, P, P, P, P]
        lib.ref_build_nodes.restype = L
        lib.ref_force.argtypes = [P, P, S, P, D, D, P, P]
        lib.ref_app_steps.argtypes = [P, P, P, S, D, D, D, I, P, P, P]
        lib.ref_decode_morton.argtypes = [P, S, D, P]
        self.lib = lib

    def decode_morton(self, keys, size):
        keys = np.ascontiguousarray(keys, np.uint64)
        out = np.zeros((len(keys), 3))
        self.lib.ref_decode_morton(_p(keys), len(keys), size, _p(out))
        return out

    def bounds(self, pos):
        pos = _f64(pos, 3)
        c = np.zeros(3)
        s = np.zeros(1)
        self.lib.ref_bounds(_p(pos), len(pos), _p(c), _p(s))
        return c, float(s[0])

    def morton_keys(self, pos, size):
        pos = _f64(pos, 3)
        k = np.zeros(len(pos), np.uint64)
        self.lib.ref_morton_keys(_p(pos), len(pos), size, _p(k))
        return k

    def sort_perm(self, keys):
        keys = np.ascontiguousarray(keys, np.uint64)
        perm = np.zeros(len(keys), np.uint32)
        self.lib.ref_sort_bodies(_p(keys), len(keys), _p(perm))
        return perm

    def guard(self, pos, center, edge):
        pos = _f64(pos, 3)
        c = _f64(center)
        return int(self.lib.ref_guard(_p(pos), len(pos), _p(c), edge))

    def build(self, pos, mass, center, edge):
        pos = _f64(pos, 3)
        mass = _f64(mass)
        c = _f64(center)
        n = len(pos)
        cap = 22 * n + 8
        keys = np.zeros(cap, np.uint64)
        counts = np.zeros(cap, np.int64)
        m = np.zeros(cap)
        com = np.zeros((cap, 3))
        cb = np.zeros(cap, np.uint8)
        q = np.zeros((cap, 6))
        box = np.zeros((cap, 4))
        got = self.lib.ref_build_nodes(_p(pos), _p(mass), n, _p(c), edge, cap, _p(keys), _p(counts), _p(m), _p(com),
                                       _p(cb), _p(q), _p(box))
        if got < 0:
            raise ValueError("REF-LITERAL refused the input (duplicate depth-21 cells)")
        return dict(keys=keys[:got], counts=counts[:got], mass=m[:got], com=com[:got], child_byte=cb[:got],
                    quad=q[:got], box=box[:got])

    def force(self, pos, mass, center, edge, theta):
        """Accelerations with the reference's fixed softening 0.025, and list lengths."""
        pos = _f64(pos, 3)
        mass = _f64(mass)
        c = _f64(center)
        acc = np.zeros((len(pos), 3))
        ll = np.zeros(len(pos), np.int64)
        rc = self.lib.ref_force(_p(pos), _p(mass), len(pos), _p(c), edge, theta, _p(acc), _p(ll))
        if rc != 0:
            raise ValueError("REF-LITERAL refused the input (duplicate depth-21 cells)")
        return acc, ll

    def app_steps(self, pos, vel, mass, acc, dt, theta, edge_factor, nsteps):
        pos = _f64(pos, 3).copy()
        vel = _f64(vel, 3).copy()
        mass = _f64(mass).copy()
        acc = _f64(acc, 3).copy()
        stage = np.zeros(6)
        perm = np.zeros(len(pos), np.uint32)
        rc = self.lib.ref_app_steps(_p(pos), _p(vel), _p(mass), len(pos), dt, theta, edge_factor, nsteps, _p(acc),
                                    _p(stage), _p(perm))
        return dict(pos=pos, vel=vel, mass=mass, acc=acc, perm=perm, stage_s=stage, rc=rc)


class RefScene:
    """The reference's own SetupSolarSystem and parseHorizonsFilez (REF-LITERAL)."""

    def __init__(self, path=REF_SCENE_LIB):
        if not os.path.exists(path):
            raise RuntimeError(f"REF-LITERAL scene library not built: {path}")
        lib = ctypes.CDLL(path)
        lib.ref_solar_system.argtypes = [ctypes.c_uint64, S, P]
        lib.ref_parse_horizons.argtypes = [ctypes.c_char_p, P, I]
        lib.ref_parse_horizons.restype = I
        self.lib = lib

    def solar_system(self, seed, n):
        out = np.zeros((n, 7))
        self.lib.ref_solar_system(seed, n, _p(out))
        return out

    def parse_horizons(self, path):
        """(count, 7) rows julianDate, position, velocity as the reference parses them."""
        cap = 1 << 16
        out = np.zeros((cap, 7))
        cnt = self.lib.ref_parse_horizons(os.fsencode(path), _p(out), cap)
        return out[:min(cnt, cap)].copy()


def relerr(a, b):
    """Per-body relative error |a - b| / |b| of (n, 3) vectors."""
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
