"""ctypes binding of libbhgpu's C ABI (include/bhgpu.h), used by the tests and bench.py.

The product is the C library; this module only loads it and converts numpy arrays. It never
computes anything itself: if libbhgpu.so is missing or a call fails, it raises.

Reference interface each method mirrors (paths relative to the reference project root):
    Simulation.bounds()        OctantBounds::OctantBounds(Body*, size_t)   src/OctantUtils.cpp:27-59
    Simulation.morton_keys()   computeMortonKey                            src/MortonKeys.hpp:137-181
    Simulation.sort_bodies()   RadixSortBodies                             src/Body.hpp:275-302
    Simulation.build()         buildLinearHashedOctreeInPlace              src/HashedOctree.hpp:211-244
    Simulation.lookup()        LinearHashedOctree::lookUpNode              src/HashedOctree.cpp:111-115
    Simulation.force()         ResetVec3D + ComputeHOTOctreeForce          src/HashedOctree.hpp:262-273
    Simulation.kick_drift()    ComputePositionAtHalfTimeStep               src/Body.hpp:306-313
    Simulation.kick()          ComputeVelocityAndPosition                  src/Body.hpp:317-324
    Simulation.step()          ofApp::update + ofApp::draw per frame       src/ofApp.cpp:169-177, 248-282
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbhgpu.so")

BH_MULTIPOLE_LITERAL = 0
BH_MULTIPOLE_QUADRUPOLE = 1

STATUS = {
    0: "BH_OK", 1: "BH_ERR_INVALID_ARG", 2: "BH_ERR_OOM", 3: "BH_ERR_DEVICE", 4: "BH_ERR_OVERFLOW_STACK",
    5: "BH_ERR_OVERFLOW_HASH", 6: "BH_ERR_OVERFLOW_NODES", 7: "BH_ERR_TIMEOUT", 8: "BH_ERR_NO_TREE",
    9: "BH_ERR_NOT_FOUND", 10: "BH_ERR_OVERFLOW_TAPE",
}

EXPORTS = [
    "bh_status_string", "bh_create", "bh_destroy", "bh_set_bodies", "bh_set_state", "bh_get_bodies",
    "bh_num_bodies", "bh_set_bodies_ref", "bh_get_bodies_ref", "bh_compute_bounds", "bh_morton_keys",
    "bh_sort_bodies", "bh_build", "bh_tree_size", "bh_tree_nodes", "bh_node_lookup", "bh_force",
    "bh_kick_drift", "bh_kick", "bh_step", "bh_params_default", "bh_synchronize", "bh_event_record",
    "bh_event_elapsed_ms", "bh_flush_l2", "bh_host_alloc", "bh_host_free", "bh_measure_fp32_peak",
    "bh_plummer", "bh_sort_keys_static", "bh_batch_set", "bh_batch_step", "bh_adjoint_forward",
    "bh_step_backward", "bh_energy_diag", "bh_autotune_walk", "bh_set_walk_variant", "bh_plummer_device",
    "bh_batch_plummer_device", "bh_tree_boxes", "bh_save_snapshot", "bh_load_snapshot", "bh_get_stream",
    "bh_check_bounded_wait", "bh_solar_system_device", "bh_parse_horizons", "bh_step_host",
    "bh_batch_step_host", "bh_set_stream", "bh_decode_morton_keys",
]


class BHError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, code)}")


class Bounds(ctypes.Structure):
    _fields_ = [("center", ctypes.c_double * 3), ("size", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [("theta", ctypes.c_double), ("eps", ctypes.c_double), ("dt", ctypes.c_double),
                ("leaf_capacity", ctypes.c_int), ("multipole", ctypes.c_int), ("edge_factor", ctypes.c_double),
                ("acc_follows_body", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_step", ctypes.c_double), ("ms_bounds", ctypes.c_double), ("ms_morton", ctypes.c_double),
                ("ms_sort", ctypes.c_double), ("ms_kick_drift", ctypes.c_double), ("ms_sort_tree", ctypes.c_double),
                ("ms_build", ctypes.c_double), ("ms_upsweep", ctypes.c_double), ("ms_walk", ctypes.c_double),
                ("n_nodes", ctypes.c_uint64), ("n_leaves", ctypes.c_uint64),
                ("interactions_cell", ctypes.c_uint64), ("interactions_p2p", ctypes.c_uint64),
                ("max_depth", ctypes.c_uint32), ("error_flags", ctypes.c_uint32), ("steps", ctypes.c_uint32),
                ("retries", ctypes.c_uint32), ("kernel_launches", ctypes.c_uint32),
                ("walk_cell_evals", ctypes.c_uint64), ("walk_point_evals", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Energy(ctypes.Structure):
    _fields_ = [("kinetic", ctypes.c_double), ("potential", ctypes.c_double), ("total", ctypes.c_double),
                ("momentum", ctypes.c_double * 3), ("angular_momentum", ctypes.c_double * 3),
                ("mass", ctypes.c_double), ("com", ctypes.c_double * 3)]

    def as_dict(self):
        return {k: (list(getattr(self, k)) if isinstance(getattr(self, k), ctypes.Array) else getattr(self, k))
                for k, _ in self._fields_}


TUNE_MAX_VARIANTS = 12  # BH_TUNE_MAX_VARIANTS


class TuneResult(ctypes.Structure):
    _fields_ = [("variants", ctypes.c_int), ("best", ctypes.c_int),
                ("warps_per_block", ctypes.c_int * TUNE_MAX_VARIANTS),
                ("min_blocks_per_sm", ctypes.c_int * TUNE_MAX_VARIANTS),
                ("stack_depth", ctypes.c_int * TUNE_MAX_VARIANTS), ("cell_form", ctypes.c_int * TUNE_MAX_VARIANTS),
                ("registers", ctypes.c_int * TUNE_MAX_VARIANTS), ("group_size", ctypes.c_int * TUNE_MAX_VARIANTS),
                ("ms", ctypes.c_float * TUNE_MAX_VARIANTS)]

    def as_dict(self):
        k = self.variants
        return {"best": self.best,
                "variants": [{"warps_per_block": self.warps_per_block[i], "min_blocks_per_sm": self.min_blocks_per_sm[i],
                              "stack_depth": self.stack_depth[i], "cell_form": self.cell_form[i],
                              "registers": self.registers[i], "group_size": self.group_size[i], "ms": self.ms[i]}
                             for i in range(k)]}


class Node(ctypes.Structure):
    _fields_ = [("key", ctypes.c_uint64), ("count", ctypes.c_int64), ("mass", ctypes.c_double),
                ("com", ctypes.c_double * 3), ("quad", ctypes.c_double * 6), ("center", ctypes.c_double * 3),
                ("size", ctypes.c_double), ("depth", ctypes.c_int32), ("child_byte", ctypes.c_uint8)]


_lib = None


def load():
    """Loads libbhgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libbhgpu.so not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    P, S, D, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int
    sig = {
        "bh_status_string": ([I], ctypes.c_char_p),
        "bh_create": ([ctypes.POINTER(P), S, I], I),
        "bh_destroy": ([P], I),
        "bh_set_bodies": ([P, P, P, S], I),
        "bh_set_state": ([P, P, P, P, S], I),
        "bh_get_bodies": ([P, P, P, P], I),
        "bh_num_bodies": ([P, ctypes.POINTER(S)], I),
        "bh_set_bodies_ref": ([P, P, S], I),
        "bh_get_bodies_ref": ([P, P, S], I),
        "bh_compute_bounds": ([P, ctypes.POINTER(Bounds)], I),
        "bh_morton_keys": ([P, D, P], I),
        "bh_sort_bodies": ([P, P], I),
        "bh_build": ([P, P, D, I, I], I),
        "bh_tree_size": ([P, ctypes.POINTER(S)], I),
        "bh_tree_nodes": ([P, S, P, P, P, P, P, P], I),
        "bh_node_lookup": ([P, ctypes.c_uint64, ctypes.POINTER(Node)], I),
        "bh_force": ([P, D, D, P, ctypes.POINTER(Stats)], I),
        "bh_kick_drift": ([P, D], I),
        "bh_kick": ([P, D], I),
        "bh_step": ([P, ctypes.POINTER(Params), I, ctypes.POINTER(Stats)], I),
        "bh_params_default": ([ctypes.POINTER(Params)], None),
        "bh_synchronize": ([P], I),
        "bh_event_record": ([P, I], I),
        "bh_event_elapsed_ms": ([P, I, I, ctypes.POINTER(ctypes.c_float)], I),
        "bh_flush_l2": ([P], I),
        "bh_host_alloc": ([ctypes.POINTER(P), S], I),
        "bh_host_free": ([P], I),
        "bh_measure_fp32_peak": ([P, ctypes.POINTER(D)], I),
        "bh_plummer": ([ctypes.c_uint64, S, D, D, P, P, P, P], I),
        "bh_sort_keys_static": ([P, P, P, P, S, P, P], I),
        "bh_batch_set": ([P, P, P, P, S], I),
        "bh_batch_step": ([P, ctypes.POINTER(Params), I, ctypes.POINTER(Stats)], I),
        "bh_adjoint_forward": ([P, ctypes.POINTER(Params), I, I, ctypes.POINTER(Stats)], I),
        "bh_step_backward": ([P, P, P, P, P, P, ctypes.POINTER(Stats)], I),
        "bh_energy_diag": ([P, D, D, ctypes.POINTER(Energy), P], I),
        "bh_autotune_walk": ([P, D, D, I, ctypes.POINTER(TuneResult)], I),
        "bh_set_walk_variant": ([P, I], I),
        "bh_plummer_device": ([P, ctypes.c_uint64, S, D, D, P, P], I),
        "bh_batch_plummer_device": ([P, ctypes.c_uint64, P, S, D, D], I),
        "bh_tree_boxes": ([P, S, P, P, P], I),
        "bh_save_snapshot": ([P, ctypes.c_char_p], I),
        "bh_load_snapshot": ([P, ctypes.c_char_p], I),
        "bh_get_stream": ([P, ctypes.POINTER(P), ctypes.POINTER(I)], I),
        "bh_set_stream": ([P, P], I),
        "bh_decode_morton_keys": ([P, P, S, D, P], I),
        "bh_check_bounded_wait": ([P, I, I], I),
        "bh_solar_system_device": ([P, ctypes.c_uint64, S, I], I),
        "bh_parse_horizons": ([ctypes.c_char_p, I, P, S, ctypes.POINTER(S)], I),
        "bh_step_host": ([P, ctypes.POINTER(Params), P, P, P, P, ctypes.POINTER(Stats)], I),
        "bh_batch_step_host": ([P, ctypes.POINTER(Params), P, P, P, P, ctypes.POINTER(Stats)], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def check(code, where):
    if code != 0:
        raise BHError(code, where)


def plummer(seed, n, a=1.0, mtot=1.0, pos_offset=None, vel_offset=None):
    """Plummer sphere (host generator of the library): returns (pos_m (n,4) f32, vel (n,4) f32)."""
    lib = load()
    pm = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    po = None if pos_offset is None else np.asarray(pos_offset, np.float64)
    vo = None if vel_offset is None else np.asarray(vel_offset, np.float64)
    check(lib.bh_plummer(seed, n, a, mtot, _ptr(po), _ptr(vo), _ptr(pm), _ptr(v)), "bh_plummer")
    return pm, v


EPHEMERIS_DTYPE = np.dtype([("jd_tdb", np.float64), ("pos", np.float64, (3,)), ("vel", np.float64, (3,))])
UNITS_SI, UNITS_GRAVITATIONAL = 0, 1
HORIZONS_LITERAL = 1


def parse_horizons(path, literal=False):
    """Records of a NASA JPL Horizons vector table (bh_parse_horizons): a structured array with
    fields jd_tdb, pos (km) and vel (km/s). literal=True applies the reference's token rule."""
    lib = load()
    cnt = ctypes.c_size_t(0)
    flags = HORIZONS_LITERAL if literal else 0
    check(lib.bh_parse_horizons(os.fsencode(path), flags, None, 0, ctypes.byref(cnt)), "bh_parse_horizons")
    out = np.zeros(cnt.value, EPHEMERIS_DTYPE)
    if cnt.value:
        check(lib.bh_parse_horizons(os.fsencode(path), flags, _ptr(out), cnt.value, ctypes.byref(cnt)),
              "bh_parse_horizons")
    return out


def bodies_from_ephemerides(tables, masses, record=0):
    """Initial bodies from Horizons tables (one table per body, record `record` of each): SI
    units (m, m/s, kg) as float32 (pos_m (k,4), vel (k,4))."""
    pm = np.zeros((len(tables), 4), np.float32)
    vel = np.zeros((len(tables), 4), np.float32)
    for k, (t, m) in enumerate(zip(tables, masses)):
        pm[k, :3] = t["pos"][record] * 1e3
        pm[k, 3] = m
        vel[k, :3] = t["vel"][record] * 1e3
    return pm, vel


def two_spheres(seed, n):
    """Clustered workload: sphere A (n/2 bodies, a = 1, M = 1, at rest at the origin) and
    sphere B (n/2 bodies, a = 0.1, M = 0.1, at (+10, 0, 0) moving with (-0.3, 0.1, 0))."""
    na = n // 2
    pa, va = plummer(seed, na, 1.0, 1.0)
    pb, vb = plummer(seed + 1, n - na, 0.1, 0.1, (10.0, 0.0, 0.0), (-0.3, 0.1, 0.0))
    return np.concatenate([pa, pb]), np.concatenate([va, vb])


def default_params(**kw):
    p = Params()
    load().bh_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Simulation:
    """One libbhgpu context (one GPU, one stream)."""

    def __init__(self, capacity, device=0):
        lib = load()
        self.lib = lib
        h = ctypes.c_void_p()
        check(lib.bh_create(ctypes.byref(h), capacity, device), "bh_create")
        self.h = h
        self.capacity = capacity

    def close(self):
        if self.h:
            self.lib.bh_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        v = ctypes.c_size_t()
        check(self.lib.bh_num_bodies(self.h, ctypes.byref(v)), "bh_num_bodies")
        return v.value

    def set_bodies(self, pos_m, vel, acc=None):
        pos_m = np.ascontiguousarray(pos_m, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        assert pos_m.shape[1] == 4 and vel.shape == pos_m.shape
        if acc is not None:
            acc = np.ascontiguousarray(acc, np.float32)
            check(self.lib.bh_set_state(self.h, _ptr(pos_m), _ptr(vel), _ptr(acc), len(pos_m)), "bh_set_state")
        else:
            check(self.lib.bh_set_bodies(self.h, _ptr(pos_m), _ptr(vel), len(pos_m)), "bh_set_bodies")

    def get_bodies(self):
        n = self.n
        p = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 4), np.float32)
        a = np.zeros((n, 4), np.float32)
        check(self.lib.bh_get_bodies(self.h, _ptr(p), _ptr(v), _ptr(a)), "bh_get_bodies")
        return p, v, a

    def bounds(self):
        b = Bounds()
        check(self.lib.bh_compute_bounds(self.h, ctypes.byref(b)), "bh_compute_bounds")
        return np.array(b.center[:]), b.size

    def morton_keys(self, size):
        k = np.zeros(self.n, np.uint64)
        check(self.lib.bh_morton_keys(self.h, size, _ptr(k)), "bh_morton_keys")
        return k

    def decode_morton_keys(self, keys, size):
        """decodeMortonKey for each key (bh_decode_morton_keys): (n, 3) float64 positions."""
        keys = np.ascontiguousarray(keys, np.uint64)
        out = np.zeros((len(keys), 3))
        check(self.lib.bh_decode_morton_keys(self.h, _ptr(keys), len(keys), size, _ptr(out)),
              "bh_decode_morton_keys")
        return out

    def sort_bodies(self):
        perm = np.zeros(self.n, np.uint32)
        check(self.lib.bh_sort_bodies(self.h, _ptr(perm)), "bh_sort_bodies")
        return perm

    def build(self, center, edge, leaf_capacity=1, multipole=BH_MULTIPOLE_QUADRUPOLE):
        c = np.ascontiguousarray(center, np.float64)
        check(self.lib.bh_build(self.h, _ptr(c), edge, leaf_capacity, multipole), "bh_build")

    def tree_size(self):
        m = ctypes.c_size_t()
        check(self.lib.bh_tree_size(self.h, ctypes.byref(m)), "bh_tree_size")
        return m.value

    def tree_nodes(self):
        m = self.tree_size()
        keys = np.zeros(m, np.uint64)
        counts = np.zeros(m, np.int64)
        mass = np.zeros(m)
        com = np.zeros((m, 3))
        cb = np.zeros(m, np.uint8)
        q = np.zeros((m, 6))
        check(self.lib.bh_tree_nodes(self.h, m, _ptr(keys), _ptr(counts), _ptr(mass), _ptr(com), _ptr(cb), _ptr(q)),
              "bh_tree_nodes")
        return dict(keys=keys, counts=counts, mass=mass, com=com, child_byte=cb, quad=q)

    def lookup(self, key):
        nd = Node()
        check(self.lib.bh_node_lookup(self.h, int(key), ctypes.byref(nd)), "bh_node_lookup")
        return nd

    def force(self, theta, eps, stats=False):
        a = np.zeros((self.n, 4), np.float32)
        st = Stats()
        check(self.lib.bh_force(self.h, theta, eps, _ptr(a), ctypes.byref(st)), "bh_force")
        return (a, st) if stats else a

    def kick_drift(self, dt):
        check(self.lib.bh_kick_drift(self.h, dt), "bh_kick_drift")

    def kick(self, dt):
        check(self.lib.bh_kick(self.h, dt), "bh_kick")

    def step(self, params, nsteps=1, stats=True):
        st = Stats()
        check(self.lib.bh_step(self.h, ctypes.byref(params), nsteps, ctypes.byref(st) if stats else None),
              "bh_step")
        return st

    def step_host(self, params, pos_in, vel_in, pos_out, vel_out, stats=True):
        """One step with host copies (bh_step_host): numpy (n, 4) float32 arrays (or None);
        page-locked arrays (PinnedArray.array) let the copies overlap the step."""
        st = Stats()
        args = []
        for a in (pos_in, vel_in, pos_out, vel_out):
            if a is not None:
                assert a.dtype == np.float32 and a.flags.c_contiguous and a.shape == (self.n, 4)
            args.append(_ptr(a))
        check(self.lib.bh_step_host(self.h, ctypes.byref(params), *args, ctypes.byref(st) if stats else None),
              "bh_step_host")
        return st

    def batch_step_host(self, params, pos_in, vel_in, pos_out, vel_out, stats=True):
        """One batched step with host copies (bh_batch_step_host); arrays as in step_host."""
        st = Stats()
        args = []
        for a in (pos_in, vel_in, pos_out, vel_out):
            if a is not None:
                assert a.dtype == np.float32 and a.flags.c_contiguous and a.shape == (self.n, 4)
            args.append(_ptr(a))
        check(self.lib.bh_batch_step_host(self.h, ctypes.byref(params), *args, ctypes.byref(st) if stats else None),
              "bh_batch_step_host")
        return st

    def batch_set(self, pos_m, vel, offsets):
        """Uploads an ensemble: system s owns rows offsets[s]:offsets[s + 1]."""
        pos_m = np.ascontiguousarray(pos_m, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        off = np.ascontiguousarray(offsets, np.uint32)
        check(self.lib.bh_batch_set(self.h, _ptr(pos_m), _ptr(vel), _ptr(off), len(off) - 1), "bh_batch_set")

    def batch_step(self, params, nsteps=1, stats=True):
        st = Stats()
        check(self.lib.bh_batch_step(self.h, ctypes.byref(params), nsteps, ctypes.byref(st) if stats else None),
              "bh_batch_step")
        return st

    def autotune(self, theta, eps, trials=3):
        """Times the walk's launch shapes on the current tree and keeps the fastest (bh_autotune_walk)."""
        r = TuneResult()
        check(self.lib.bh_autotune_walk(self.h, theta, eps, trials, ctypes.byref(r)), "bh_autotune_walk")
        return r.as_dict()

    def plummer_device(self, seed, n, a=1.0, mtot=1.0, pos_offset=None, vel_offset=None):
        """Generates a Plummer sphere on the device as the context's state (bh_plummer_device)."""
        po = None if pos_offset is None else np.ascontiguousarray(pos_offset, np.float64)
        vo = None if vel_offset is None else np.ascontiguousarray(vel_offset, np.float64)
        check(self.lib.bh_plummer_device(self.h, seed, n, a, mtot, _ptr(po), _ptr(vo)), "bh_plummer_device")

    def solar_system_device(self, seed, n, units=UNITS_SI):
        """Generates the reference app's solar-system scene on the device (bh_solar_system_device)."""
        check(self.lib.bh_solar_system_device(self.h, seed, n, units), "bh_solar_system_device")

    def batch_plummer_device(self, seed, offsets, a=1.0, mtot=1.0):
        """Generates an ensemble of Plummer spheres on the device (bh_batch_plummer_device)."""
        off = np.ascontiguousarray(offsets, np.uint32)
        check(self.lib.bh_batch_plummer_device(self.h, seed, _ptr(off), len(off) - 1, a, mtot),
              "bh_batch_plummer_device")

    def tree_boxes(self):
        m = self.tree_size()
        box = np.zeros((m, 4), np.float32)
        depth = np.zeros(m, np.int32)
        count = np.zeros(m, np.int64)
        check(self.lib.bh_tree_boxes(self.h, m, _ptr(box), _ptr(depth), _ptr(count)), "bh_tree_boxes")
        return box, depth, count

    def save_snapshot(self, path):
        check(self.lib.bh_save_snapshot(self.h, os.fsencode(path)), "bh_save_snapshot")

    def load_snapshot(self, path):
        check(self.lib.bh_load_snapshot(self.h, os.fsencode(path)), "bh_load_snapshot")

    def set_walk_variant(self, v):
        check(self.lib.bh_set_walk_variant(self.h, v), "bh_set_walk_variant")

    def energy(self, theta, eps, potential=False):
        """Conservation diagnostics of the current state over the current tree (bh_energy_diag)."""
        e = Energy()
        pot = np.zeros(self.n, np.float32) if potential else None
        check(self.lib.bh_energy_diag(self.h, theta, eps, ctypes.byref(e), _ptr(pot)), "bh_energy_diag")
        return (e.as_dict(), pot) if potential else e.as_dict()

    def adjoint_forward(self, params, nsteps, checkpoint_every, stats=True):
        """Differentiable trajectory: nsteps KDK steps in upload order with checkpoints."""
        st = Stats()
        check(self.lib.bh_adjoint_forward(self.h, ctypes.byref(params), nsteps, checkpoint_every,
                                          ctypes.byref(st) if stats else None), "bh_adjoint_forward")
        return st

    def step_backward(self, dl_dpos, dl_dvel, stats=False):
        """Gradients (d pos0 (n, 4), d vel0 (n, 4), d mass (n,)) of a loss whose gradients with
        respect to the final positions / velocities are dl_dpos / dl_dvel ((n, 3) or (n, 4), or None)."""
        def as4(a):
            if a is None:
                return None
            a = np.asarray(a, np.float32)
            out = np.zeros((self.n, 4), np.float32)
            out[:, :3] = a[:, :3]
            return out
        gx = np.zeros((self.n, 4), np.float32)
        gv = np.zeros((self.n, 4), np.float32)
        gm = np.zeros(self.n, np.float32)
        st = Stats()
        bx, bv = as4(dl_dpos), as4(dl_dvel)  # kept alive across the call
        check(self.lib.bh_step_backward(self.h, _ptr(bx), _ptr(bv), _ptr(gx), _ptr(gv), _ptr(gm), ctypes.byref(st)),
              "bh_step_backward")
        return (gx, gv, gm, st) if stats else (gx, gv, gm)

    def synchronize(self):
        check(self.lib.bh_synchronize(self.h), "bh_synchronize")

    def event_record(self, slot):
        check(self.lib.bh_event_record(self.h, slot), "bh_event_record")

    def event_elapsed_ms(self, a, b):
        ms = ctypes.c_float()
        check(self.lib.bh_event_elapsed_ms(self.h, a, b, ctypes.byref(ms)), "bh_event_elapsed_ms")
        return ms.value

    def flush_l2(self):
        check(self.lib.bh_flush_l2(self.h), "bh_flush_l2")

    def fp32_peak_tflops(self):
        v = ctypes.c_double()
        check(self.lib.bh_measure_fp32_peak(self.h, ctypes.byref(v)), "bh_measure_fp32_peak")
        return v.value


class PinnedArray:
    """numpy view of pinned host memory allocated by bh_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        self.lib = load()
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = ctypes.c_void_p()
        check(self.lib.bh_host_alloc(ctypes.byref(p), nbytes), "bh_host_alloc")
        self.p = p
        buf = (ctypes.c_char * nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.p:
            self.array = None
            self.lib.bh_host_free(self.p)
            self.p = None
