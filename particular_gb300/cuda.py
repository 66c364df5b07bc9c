"""The `cuda` compute methods: the GB300 counterpart of particular's `gpu` module.

Mirrors particular/src/gpu/mod.rs:
* CudaResources      - GpuResources (gpu/mod.rs:84-143): create once, reuse across calls
* BruteForce         - gpu::BruteForce (gpu/mod.rs:145-208): `compute(storage)`
* BarnesHut          - the GPU counterpart of sequential::BarnesHut (sequential.rs:432-543)
* cuda_brute_force / cuda_barnes_hut - the GpuCompute::gpu_brute_force sugar (gpu/mod.rs:13-37)

`compute` accepts every storage the reference's methods accept (a particle
sequence, Ordered, Reordered, Between) and returns the accelerations of the
affected particles as a float32 (n, 3) array, in the affected order (the
reference returns a `std::vec::IntoIter` over the same values).
"""
import ctypes

import numpy as np

from . import _native as N
from .gravity import fields, positions
from .storage import as_between


class CudaResources:
    """A libparticular_cuda context: device, stream and grow-only device buffers."""

    def __init__(self, device=0):
        L = N.lib()
        h = ctypes.c_void_p()
        N.check(L.pt_ctx_create(ctypes.byref(h), int(device)))
        self._h = h
        self.device = int(device)

    @property
    def handle(self):
        if self._h is None:
            raise N.CudaError(N.PT_ERR_INVALID, "CudaResources used after close()")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            N.lib().pt_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def launch_count(self):
        return int(N.lib().pt_ctx_launch_count(self.handle))

    @property
    def device_bytes(self):
        return int(N.lib().pt_ctx_device_bytes(self.handle))

    @property
    def sm_count(self):
        return int(N.lib().pt_ctx_sm_count(self.handle))

    def set_capacity_limit(self, nbytes):
        N.check(N.lib().pt_ctx_set_capacity_limit(self.handle, int(nbytes)))

    def set_stream(self, stream_handle):
        """Enqueue on a raw cudaStream_t (int handle); None = the context's own stream."""
        N.check(N.lib().pt_ctx_set_stream(self.handle, stream_handle or None))

    def synchronize(self):
        N.check(N.lib().pt_ctx_synchronize(self.handle))


def _ptr(a):
    return a.ctypes.data if a.size else None


class BruteForce:
    """cuda::BruteForce: all-pairs accelerations on the GPU.

    `exact=True` selects the bit-identical restatement of sequential::BruteForce
    (sequential j order, IEEE sqrt and divide); the default is the fast FP32 path
    with compensated accumulation. `dvec3=True` computes over glam DVec3 bodies:
    float64 in and out, the reference's f64 kernel bit for bit (storages built with
    dtype=np.float64 keep their float64 values).
    """

    def __init__(self, resources, interaction, exact=False, vec3a=False, dvec3=False):
        self.resources = resources
        self.interaction = interaction
        self.exact = bool(exact)
        self.vec3a = bool(vec3a)  # glam Vec3A/Vec4 operand order (exact path)
        self.dvec3 = bool(dvec3)

    def load_tree(self, internal, orthant, bbox, data, root=0):
        """Makes a tree the caller built (the reference's RootedOrthtree over
        GravitationalField<Vec3, f32>, flattened per node: internal flags, 8 orthant
        slots with -1 for None, bbox min/max, data (x, y, z, mass); root -1 = None) the
        resources' current tree; pass the returned DeviceTree as the affecting side of
        Between to walk it (flags 0 or group only: the tree carries monopoles)."""
        internal = np.ascontiguousarray(internal, np.uint8)
        n = internal.shape[0]
        orthant = np.ascontiguousarray(orthant, np.int32).reshape(n, 8)
        bbox = np.ascontiguousarray(bbox, np.float32).reshape(n, 6)
        data = np.ascontiguousarray(data, np.float32).reshape(n, 4)
        g = ctypes.c_uint64(0)
        N.check(N.lib().pt_bh_load_tree(self.resources.handle, _ptr(orthant), _ptr(bbox), _ptr(internal),
                                        _ptr(data), n, int(root), ctypes.byref(g)))
        return DeviceTree(self.resources, n, g.value)

    def compute(self, storage):
        b = as_between(storage)
        if self.dvec3:
            aff = positions(b.affected, np.float64)
            src = fields(b.affecting, np.float64)
            out = np.zeros((aff.shape[0], 3), np.float64)
            if aff.shape[0] == 0:
                return out
            same = b.affected is b.affecting
            it = self.interaction
            eps = getattr(it, "softening64", it.softening)
            N.check(N.lib().pt_bf_accel_dvec3(self.resources.handle, _ptr(aff), aff.shape[0],
                                              _ptr(aff) if same else _ptr(src), src.shape[0],
                                              eps, int(it.is_checked), _ptr(out)))
            return out
        aff = positions(b.affected)
        src = fields(b.affecting)
        out = np.zeros((aff.shape[0], 3), np.float32)
        if aff.shape[0] == 0:
            return out
        same = b.affected is b.affecting
        it = self.interaction
        flags = (N.PT_BF_EXACT if self.exact else 0) | (N.PT_BF_VEC3A if self.vec3a else 0)
        N.check(N.lib().pt_bf_accel_f32(self.resources.handle, _ptr(aff), aff.shape[0],
                                        _ptr(aff) if same else _ptr(src), src.shape[0],
                                        it.softening, int(it.is_checked), flags, _ptr(out)))
        return out


def cuda_brute_force(storage, resources, interaction, exact=False):
    """`storage.cuda_brute_force(resources, interaction)` (CudaCompute sugar)."""
    return BruteForce(resources, interaction, exact).compute(storage)


class DeviceTree:
    """A Barnes-Hut tree kept on the device (the counterpart of a RootedOrthtree built
    once and reused through Between(affected, &tree): particular/src/lib.rs:186-199).
    It stays valid until the next Barnes-Hut call on the same CudaResources replaces
    the context's tree; using it afterwards raises."""

    def __init__(self, resources, n_affecting, generation):
        self.resources = resources
        self.n_affecting = int(n_affecting)
        self.generation = int(generation)

    def is_current(self):
        g = ctypes.c_uint64(0)
        N.check(N.lib().pt_bh_tree_generation(self.resources.handle, ctypes.byref(g)))
        return g.value == self.generation


class BarnesHut:
    """cuda::BarnesHut { theta }: the reference's orthtree built on the GPU every call
    and walked with the reference's opening rule (sequential.rs:466-505).

    quadrupole=True adds the accepted cells' quadrupole terms; group=True opens a
    cell for a warp of 64 neighbouring bodies whenever one of them opens it. Both
    only ever reduce the error relative to the reference's monopole walk.
    local=True (with group) sends nodes far from the group into a second-order
    local expansion about the group's centre (resources-wide ratio:
    pt_bh_set_local_ratio); its truncation error is judged against FP64.
    relative=alpha (with group) also opens a cell where its truncation bound
    M w^3 / d^5 (M w^2 / d^4 without quadrupoles) exceeds alpha |a|, |a| estimated
    once per group; theta stays the geometric cap. monopole=beta (with relative and
    quadrupole) evaluates an accepted cell without its quadrupole where the term it
    drops, M w^2 / d^4, stays within beta alpha |a| (pt_bh_set_relative_monopole).
    """

    def __init__(self, theta, resources, interaction, quadrupole=False, group=False,
                 learned=False, local=False, dvec3=False, relative=None, monopole=None):
        self.dvec3 = bool(dvec3)  # glam DVec3 bodies: the f64 method (reference rule only)
        self.theta64 = float(theta)
        self.theta = float(np.float32(theta))
        self.resources = resources
        self.interaction = interaction
        self.quadrupole = bool(quadrupole)
        self.group = bool(group)
        self.learned = bool(learned)  # needs a model (particular_gb300.learned) and group
        self.local = bool(local)      # far nodes through the group's local expansion
        self.relative = None if relative is None else float(relative)  # error-bound factor alpha
        # with relative and quadrupole: cells whose quadrupole term stays within
        # monopole x alpha |a| are evaluated without it (None: the resources' setting)
        self.monopole = None if monopole is None else float(monopole)

    @property
    def flags(self):
        return ((N.PT_BH_QUADRUPOLE if self.quadrupole else 0) | (N.PT_BH_GROUP if self.group else 0)
                | (N.PT_BH_LEARNED if self.learned else 0) | (N.PT_BH_LOCAL if self.local else 0)
                | (N.PT_BH_RELATIVE if self.relative is not None else 0))

    def _set_alpha(self):
        if self.relative is not None:
            N.check(N.lib().pt_bh_set_relative_alpha(self.resources.handle, self.relative))
        if self.monopole is not None:
            N.check(N.lib().pt_bh_set_relative_monopole(self.resources.handle, self.monopole))

    def build(self, affecting):
        """Builds the tree over `affecting` (any storage of particles) once; pass the
        returned DeviceTree as the affecting side of Between to walk it."""
        src = fields(affecting)
        g = ctypes.c_uint64(0)
        N.check(N.lib().pt_bh_build(self.resources.handle, _ptr(src), src.shape[0], ctypes.byref(g)))
        return DeviceTree(self.resources, src.shape[0], g.value)

    def load_tree(self, internal, orthant, bbox, data, root=0):
        """Makes a tree the caller built (the reference's RootedOrthtree over
        GravitationalField<Vec3, f32>, flattened per node: internal flags, 8 orthant
        slots with -1 for None, bbox min/max, data (x, y, z, mass); root -1 = None) the
        resources' current tree; pass the returned DeviceTree as the affecting side of
        Between to walk it (flags 0 or group only: the tree carries monopoles)."""
        internal = np.ascontiguousarray(internal, np.uint8)
        n = internal.shape[0]
        orthant = np.ascontiguousarray(orthant, np.int32).reshape(n, 8)
        bbox = np.ascontiguousarray(bbox, np.float32).reshape(n, 6)
        data = np.ascontiguousarray(data, np.float32).reshape(n, 4)
        g = ctypes.c_uint64(0)
        N.check(N.lib().pt_bh_load_tree(self.resources.handle, _ptr(orthant), _ptr(bbox), _ptr(internal),
                                        _ptr(data), n, int(root), ctypes.byref(g)))
        return DeviceTree(self.resources, n, g.value)

    def compute(self, storage):
        b = as_between(storage)
        if self.dvec3:
            if self.flags:
                raise N.CudaError(N.PT_ERR_INVALID, "the f64 method is the reference rule: no flags")
            aff = positions(b.affected, np.float64)
            src = fields(b.affecting, np.float64)
            out = np.zeros((aff.shape[0], 3), np.float64)
            if aff.shape[0] == 0:
                return out
            same = b.affected is b.affecting
            it = self.interaction
            N.check(N.lib().pt_bh_accel_dvec3(self.resources.handle, _ptr(aff), aff.shape[0],
                                              _ptr(aff) if same else _ptr(src), src.shape[0], self.theta64,
                                              getattr(it, "softening64", it.softening), 0, _ptr(out)))
            return out
        if isinstance(b.affecting, DeviceTree):
            tree = b.affecting
            if tree.resources is not self.resources:
                raise ValueError("the tree belongs to another CudaResources")
            if not tree.is_current():
                raise N.CudaError(N.PT_ERR_INVALID, "the tree was replaced by a later Barnes-Hut call")
            aff = positions(b.affected)
            out = np.zeros((aff.shape[0], 3), np.float32)
            self._set_alpha()
            if aff.shape[0]:
                N.check(N.lib().pt_bh_walk(self.resources.handle, _ptr(aff), aff.shape[0], self.theta,
                                           self.interaction.softening, self.flags, _ptr(out)))
            return out
        aff = positions(b.affected)
        src = fields(b.affecting)
        out = np.zeros((aff.shape[0], 3), np.float32)
        if aff.shape[0] == 0:
            return out
        same = b.affected is b.affecting
        self._set_alpha()
        N.check(N.lib().pt_bh_accel_f32(self.resources.handle, _ptr(aff), aff.shape[0],
                                        _ptr(aff) if same else _ptr(src), src.shape[0], self.theta,
                                        self.interaction.softening, self.flags, _ptr(out)))
        return out

    def stats(self):
        """Counters of the last Barnes-Hut call on these resources (pt_bh_last_stats)."""
        st = N.BhStats()
        N.check(N.lib().pt_bh_last_stats(self.resources.handle, ctypes.byref(st)))
        return {k: int(getattr(st, k)) for k, _ in N.BhStats._fields_}

    def export_tree_dvec3(self):
        """The last f64 tree in preorder: com_mass (n, 4), links (n, 4), centre_width (n, 4)."""
        n = self.stats()["nodes"]
        cm = np.zeros((n, 4), np.float64)
        ln = np.zeros((n, 4), np.int32)
        cw = np.zeros((n, 4), np.float64)
        N.check(N.lib().pt_bh_export_tree_dvec3(self.resources.handle, _ptr(cm), _ptr(ln), _ptr(cw), n))
        return {"com_mass": cm, "links": ln, "centre_width": cw, "width": cw[:, 3]}

    def export_tree(self):
        """The last tree in preorder: com_mass (n, 4), links (n, 4) int32, quad (n, 8)."""
        st = self.stats()
        n = st["nodes"]
        cm = np.zeros((n, 4), np.float32)
        ln = np.zeros((n, 4), np.int32)
        q = np.zeros((n, 8), np.float32)
        N.check(N.lib().pt_bh_export_tree(self.resources.handle, _ptr(cm), _ptr(ln), _ptr(q), n))
        return {"com_mass": cm, "links": ln, "quad": q, "width": ln[:, 0].view(np.float32)}


def cuda_barnes_hut(storage, theta, resources, interaction, **kw):
    """`storage.cuda_barnes_hut(theta, resources, interaction)` (CudaCompute sugar)."""
    return BarnesHut(theta, resources, interaction, **kw).compute(storage)


class Leapfrog:
    """Kick-drift-kick leapfrog around a cuda method (the driver the reference's tests
    and benchmark write by hand around their methods; particular/benches/benchmark.rs:81).

    `method` is a BruteForce or BarnesHut instance; `run` advances host state in place.
    """

    def __init__(self, method, dt):
        self.method = method
        self.dt = float(np.float32(dt))

    def _args(self):
        m = self.method
        if isinstance(m, BarnesHut):
            m._set_alpha()  # the method's error-bound factor, when it uses one
            return N.PT_METHOD_BARNES_HUT, m.theta, m.interaction.softening, m.flags
        return (N.PT_METHOD_BRUTE_FORCE, 0.0, m.interaction.softening,
                N.PT_BF_EXACT if m.exact else 0)

    def run(self, bodies, vel, steps):
        """bodies: (n, 4) float32 (x, y, z, mu); vel: (n, 3) or (n, 4) float32.
        Returns the advanced (bodies, vel) as new arrays."""
        b = np.ascontiguousarray(bodies, np.float32).copy()
        v4 = np.zeros((b.shape[0], 4), np.float32)
        v4[:, :3] = np.asarray(vel, np.float32)[:, :3]
        method, theta, soft, flags = self._args()
        N.check(N.lib().pt_leapfrog(self.method.resources.handle, _ptr(b), _ptr(v4), b.shape[0],
                                    self.dt, int(steps), method, theta, soft, flags))
        return b, v4[:, :3].copy()
