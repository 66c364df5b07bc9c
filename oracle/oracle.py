"""ctypes wrapper over the C oracle (test infrastructure only).

Every function takes packed float32 arrays: sources (n, 4) = (x, y, z, mu),
targets (n, 4) or (n, 3) = positions. See oracle/pt_oracle.c for the reference
file:line each restated function follows.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        L = ctypes.CDLL(path)
        L.oracle_bf_f32.argtypes = [_f32p, ctypes.c_size_t, _f32p, ctypes.c_size_t,
                                    ctypes.c_float, ctypes.c_int, _f32p, ctypes.c_int]
        L.oracle_bf_f32_vec3a.argtypes = [_f32p, ctypes.c_size_t, _f32p, ctypes.c_size_t,
                                          ctypes.c_float, ctypes.c_int, _f32p, ctypes.c_int]
        L.oracle_bf_f64.argtypes = [_f32p, ctypes.c_size_t, _f32p, ctypes.c_size_t,
                                    ctypes.c_double, ctypes.c_int, _f64p, ctypes.c_int]
        L.oracle_bf_dvec3.argtypes = [_f64p, ctypes.c_size_t, _f64p, ctypes.c_size_t,
                                      ctypes.c_double, ctypes.c_int, _f64p, ctypes.c_int]
        L.oracle_bf_pairs_f32.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_float, _f32p]
        L.oracle_bf_pairs_f64.argtypes = [_f64p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_double, _f64p]
        L.oracle_bh_build.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_int]
        L.oracle_bh_build.restype = ctypes.c_void_p
        L.oracle_tree_free.argtypes = [ctypes.c_void_p]
        L.oracle_tree_node_count.argtypes = [ctypes.c_void_p]
        L.oracle_tree_node_count.restype = ctypes.c_size_t
        L.oracle_tree_max_depth.argtypes = [ctypes.c_void_p]
        L.oracle_tree_export.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 6
        L.oracle_bh_walk.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_int, _f32p, _u32p, ctypes.c_int]
        L.oracle_bh_walk_sum64.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_int, _f64p, _f64p, ctypes.c_int]
        L.oracle_bh_f32.argtypes = [_f32p, ctypes.c_size_t, _f32p, ctypes.c_size_t,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int, _f32p, _u32p,
                                    ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_bh_dvec3.argtypes = [_f64p, ctypes.c_size_t, _f64p, ctypes.c_size_t,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int, _f64p, _u32p,
                                      ctypes.c_int]
        L.oracle_bh_build_dvec3.argtypes = [_f64p, ctypes.c_size_t, ctypes.c_int]
        L.oracle_bh_build_dvec3.restype = ctypes.c_void_p
        L.oracle_tree_free_dvec3.argtypes = [ctypes.c_void_p]
        L.oracle_tree_node_count_dvec3.argtypes = [ctypes.c_void_p]
        L.oracle_tree_node_count_dvec3.restype = ctypes.c_size_t
        L.oracle_tree_max_depth_dvec3.argtypes = [ctypes.c_void_p]
        L.oracle_tree_export_dvec3.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 6
        _lib = L
    return _lib


def _targets(a):
    a = np.asarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] not in (3, 4):
        raise ValueError("targets must be (n, 3) or (n, 4)")
    if a.shape[1] == 3:
        a = np.concatenate([a, np.zeros((a.shape[0], 1), np.float32)], axis=1)
    return np.ascontiguousarray(a)


def _sources(s):
    s = np.ascontiguousarray(np.asarray(s, dtype=np.float32))
    if s.ndim != 2 or s.shape[1] != 4:
        raise ValueError("sources must be (n, 4) = (x, y, z, mu)")
    return s


def max_threads():
    return lib().oracle_max_threads()


def bf_f32(targets, sources, softening=0.0, checked=True, threads=0):
    """sequential::BruteForce / parallel::BruteForce (bit-identical per body)."""
    t, s = _targets(targets), _sources(sources)
    out = np.zeros((t.shape[0], 3), np.float32)
    rc = lib().oracle_bf_f32(t, t.shape[0], s, s.shape[0], softening, int(checked), out, threads)
    if rc:
        raise RuntimeError(f"oracle_bf_f32 failed: {rc}")
    return out


def bf_f32_vec3a(targets, sources, softening=0.0, checked=True, threads=0):
    """sequential::BruteForce with glam Vec3A/Vec4's operand order (d * m / ...)."""
    t, s = _targets(targets), _sources(sources)
    out = np.zeros((t.shape[0], 3), np.float32)
    rc = lib().oracle_bf_f32_vec3a(t, t.shape[0], s, s.shape[0], softening, int(checked), out,
                                   threads)
    if rc:
        raise RuntimeError(f"oracle_bf_f32_vec3a failed: {rc}")
    return out


def bf_f64(targets, sources, softening=0.0, checked=True, threads=0):
    """FP64 brute force of the same formula: the error judge."""
    t, s = _targets(targets), _sources(sources)
    out = np.zeros((t.shape[0], 3), np.float64)
    rc = lib().oracle_bf_f64(t, t.shape[0], s, s.shape[0], softening, int(checked), out, threads)
    if rc:
        raise RuntimeError(f"oracle_bf_f64 failed: {rc}")
    return out


def bf_dvec3(targets, sources, softening=0.0, checked=True, threads=0):
    """sequential::BruteForce over glam DVec3 bodies: double (n, 4) in, double (n, 3) out."""
    t = np.ascontiguousarray(np.asarray(targets, np.float64))
    if t.shape[1] == 3:
        t = np.ascontiguousarray(np.concatenate([t, np.zeros((t.shape[0], 1))], axis=1))
    s = np.ascontiguousarray(np.asarray(sources, np.float64))
    out = np.zeros((t.shape[0], 3), np.float64)
    rc = lib().oracle_bf_dvec3(t, t.shape[0], s, s.shape[0], softening, int(checked), out, threads)
    if rc:
        raise RuntimeError(f"oracle_bf_dvec3 failed: {rc}")
    return out


def bf_pairs(bodies, restrict_len=None, softening=0.0):
    """BruteForcePairs / RestrictedBruteForce over one slice (f32 or f64 by dtype):
    every body is affected, the first `restrict_len` (default all) are affecting."""
    b = np.ascontiguousarray(bodies)
    n = b.shape[0]
    r = n if restrict_len is None else int(restrict_len)
    if b.dtype == np.float64:
        out = np.zeros((n, 3), np.float64)
        rc = lib().oracle_bf_pairs_f64(b, n, r, softening, out)
    else:
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros((n, 3), np.float32)
        rc = lib().oracle_bf_pairs_f32(b, n, r, softening, out)
    if rc:
        raise RuntimeError(f"oracle_bf_pairs failed: {rc}")
    return out


def bh_f32(targets, sources, theta, softening=0.0, checked=True, threads=0, accepted=False):
    """sequential::BarnesHut (tree over `sources`, walk for every target)."""
    t, s = _targets(targets), _sources(sources)
    out = np.zeros((t.shape[0], 3), np.float32)
    acc = np.zeros(t.shape[0], np.uint32) if accepted else None
    rc = lib().oracle_bh_f32(t, t.shape[0], s, s.shape[0], theta, softening, int(checked), out,
                             acc.ctypes.data if accepted else None, threads)
    if rc:
        raise RuntimeError(f"oracle_bh_f32 failed: {rc}")
    return (out, acc) if accepted else out


def bh_dvec3(targets, sources, theta, softening=0.0, checked=True, threads=0, accepted=False):
    """sequential::BarnesHut over glam DVec3 bodies (double (n, 4) in, double (n, 3) out)."""
    t = np.ascontiguousarray(np.asarray(targets, np.float64))
    if t.shape[1] == 3:
        t = np.ascontiguousarray(np.concatenate([t, np.zeros((t.shape[0], 1))], axis=1))
    s = np.ascontiguousarray(np.asarray(sources, np.float64))
    out = np.zeros((t.shape[0], 3), np.float64)
    acc = np.zeros(t.shape[0], np.uint32) if accepted else None
    rc = lib().oracle_bh_dvec3(t, t.shape[0], s, s.shape[0], theta, softening, int(checked), out,
                               acc.ctypes.data if accepted else None, threads)
    if rc:
        raise RuntimeError(f"oracle_bh_dvec3 failed: {rc}")
    return (out, acc) if accepted else out


def tree_dvec3_export(sources):
    """The reference orthtree over DVec3 bodies, exported like Tree.export (double box/data)."""
    s = np.ascontiguousarray(np.asarray(sources, np.float64))
    L = lib()
    h = L.oracle_bh_build_dvec3(s, s.shape[0], 0)
    if not h:
        raise MemoryError("oracle_bh_build_dvec3 failed")
    try:
        if L.oracle_tree_max_depth_dvec3(h) < 0:
            raise RuntimeError("oracle_bh_build_dvec3: depth limit reached")
        n = L.oracle_tree_node_count_dvec3(h)
        internal = np.zeros(n, np.int32)
        child = np.zeros((n, 8), np.int32)
        box = np.zeros((n, 6), np.float64)
        data = np.zeros((n, 4), np.float64)
        rng = np.zeros((n, 2), np.int32)
        perm = np.zeros(s.shape[0], np.uint32)
        L.oracle_tree_export_dvec3(h, internal.ctypes.data, child.ctypes.data, box.ctypes.data,
                                   data.ctypes.data, rng.ctypes.data, perm.ctypes.data)
        return dict(internal=internal, child=child, box=box, data=data, range=rng, perm=perm)
    finally:
        L.oracle_tree_free_dvec3(h)


class Tree:
    """The reference orthtree built over `sources` (tree/mod.rs:91-138)."""

    def __init__(self, sources, max_depth=0):
        self._s = _sources(sources)
        self._h = lib().oracle_bh_build(self._s, self._s.shape[0], max_depth)
        if not self._h:
            raise MemoryError("oracle_bh_build failed")
        if lib().oracle_tree_max_depth(self._h) < 0:
            lib().oracle_tree_free(self._h)
            self._h = None
            raise RuntimeError("oracle_bh_build: depth limit reached")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_tree_free(self._h)
            self._h = None

    @property
    def node_count(self):
        return lib().oracle_tree_node_count(self._h)

    @property
    def max_depth(self):
        return lib().oracle_tree_max_depth(self._h)

    def export(self):
        n = self.node_count
        internal = np.zeros(n, np.int32)
        child = np.zeros((n, 8), np.int32)
        box = np.zeros((n, 6), np.float32)
        data = np.zeros((n, 4), np.float32)
        rng = np.zeros((n, 2), np.int32)
        perm = np.zeros(self._s.shape[0], np.uint32)
        lib().oracle_tree_export(self._h, internal.ctypes.data, child.ctypes.data,
                                 box.ctypes.data, data.ctypes.data, rng.ctypes.data,
                                 perm.ctypes.data)
        return dict(internal=internal, child=child, box=box, data=data, range=rng, perm=perm)

    def walk(self, targets, theta, softening=0.0, checked=True, threads=0, accepted=False):
        t = _targets(targets)
        out = np.zeros((t.shape[0], 3), np.float32)
        acc = np.zeros(t.shape[0], np.uint32) if accepted else None
        rc = lib().oracle_bh_walk(self._h, t, t.shape[0], theta, softening, int(checked), out,
                                  acc.ctypes.data if accepted else None, threads)
        if rc:
            raise RuntimeError(f"oracle_bh_walk failed: {rc}")
        return (out, acc) if accepted else out

    def walk_sum64(self, targets, theta, softening=0.0, checked=True, threads=0):
        """The same accepted set per body as walk(), its terms computed and summed in
        double: (FP64 sums, per-body sums of the terms' norms)."""
        t = _targets(targets)
        out = np.zeros((t.shape[0], 3), np.float64)
        l1 = np.zeros(t.shape[0], np.float64)
        rc = lib().oracle_bh_walk_sum64(self._h, t, t.shape[0], theta, softening, int(checked), out,
                                        l1, threads)
        if rc:
            raise RuntimeError(f"oracle_bh_walk_sum64 failed: {rc}")
        return out, l1
