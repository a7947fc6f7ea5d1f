"""GB300 (sm_103a) VortonSim velocity-from-vorticity step.

Python host side of ``libvortegrid.so`` (declared in ``include/vortegrid.h``).
It mirrors the reference's particle-operation interface for this step
(mijagourlay/VorteGrid, Samples/MjgIntelFluidDemo_Part20):

  * ``PclOpVortonSim.Operate(particles, timeStep, uFrame)`` --
    VortonFluid/pclOpVortonSim.cpp:51-71, on an array of the reference's
    96-byte ``Particle`` records (``PARTICLE_DTYPE``);
  * ``VortonSim`` -- VortonFluid/vortonSim.h:279-455: ``Update``,
    ``GetVelocityGrid``, ``GetVectorPotential``, settings as in the reference;
  * ``PclOpAssignVelocityFromFieldAndEvolve`` -- tracer advection
    (Particles/Operation/pclOpAdvect.cpp:132-152, pclOpEvolve.cpp:36-58).

There is no CPU fallback: every call goes through the CUDA library, and
importing a function that needs it raises if the library is missing.
"""
import ctypes
import os

import numpy as np

from . import workloads  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvortegrid.so")

# vg_status
OK, EMPTY, OUT_OF_GRID, NONFINITE, OOM, TIMEOUT, INVALID, CUDA_ERROR, NOT_CONVERGED, TOO_LARGE = range(10)
VELOCITY_POISSON, VELOCITY_TREE, VELOCITY_DIRECT = 0, 1, 2
NUMERICS_FAST, NUMERICS_REFERENCE = 0, 1
POISSON_MULTIGRID, POISSON_REFERENCE_CASCADE = 0, 1
WARM_ZERO, WARM_PREVIOUS, WARM_NETWORK = 0, 1, 2

# The reference's Particle record on LP64 (Particles/particle.h:425-482).
PARTICLE_DTYPE = np.dtype({
    "names": ["position", "velocity", "orientation", "angular_velocity", "density", "size", "birth_time",
              "fuel", "flame", "smoke"],
    "formats": [(np.float32, 3), (np.float32, 3), (np.float32, 3), (np.float32, 3), np.float32, np.float32,
                np.int32, np.float32, np.float32, np.float32],
    "offsets": [0, 12, 24, 36, 48, 52, 56, 60, 64, 68],
    "itemsize": 96,
})


class VgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class GridGeom(ctypes.Structure):
    _fields_ = [("min_corner", ctypes.c_float * 3), ("extent", ctypes.c_float * 3),
                ("cell_spacing", ctypes.c_float * 3), ("cells_per_extent", ctypes.c_float * 3),
                ("num_points", ctypes.c_uint * 3)]

    @property
    def points(self):
        return tuple(int(v) for v in self.num_points)

    @property
    def capacity(self):
        p = self.points
        return p[0] * p[1] * p[2]

    def as12(self):
        return np.array(list(self.min_corner) + list(self.extent) + list(self.cell_spacing) +
                        list(self.cells_per_extent), np.float32)

    @staticmethod
    def make(min_corner, extent, num_points):
        """Explicit geometry: spacing and cells-per-extent follow
        UniformGridGeometry::PrecomputeSpacing (uniformGrid.h:794-809)."""
        g = GridGeom()
        for a in range(3):
            g.min_corner[a] = float(np.float32(min_corner[a]))
            g.extent[a] = float(np.float32(extent[a]))
            g.num_points[a] = int(num_points[a])
            cells = np.float32(int(num_points[a]) - 1)
            g.cell_spacing[a] = float(np.float32(extent[a]) / cells)
            g.cells_per_extent[a] = float(cells / np.float32(extent[a]))
        return g

    @staticmethod
    def from12(g12, np3):
        g = GridGeom()
        for a in range(3):
            g.min_corner[a] = float(g12[a]); g.extent[a] = float(g12[3 + a])
            g.cell_spacing[a] = float(g12[6 + a]); g.cells_per_extent[a] = float(g12[9 + a])
            g.num_points[a] = int(np3[a])
        return g


class Particles(ctypes.Structure):
    """vg_particles: one particle group's device arrays (pointers may be 0)."""
    _fields_ = [("pos_size", ctypes.c_void_p), ("vel4", ctypes.c_void_p), ("angvel4", ctypes.c_void_p),
                ("orient4", ctypes.c_void_p), ("density", ctypes.c_void_p), ("fire4", ctypes.c_void_p),
                ("birth", ctypes.c_void_p), ("count", ctypes.c_size_t), ("capacity", ctypes.c_size_t)]


class ParticleValues(ctypes.Structure):
    """vg_particle_values: the 17 values of PclOpEmit's template and spread."""
    _fields_ = [("position", ctypes.c_float * 3), ("velocity", ctypes.c_float * 3),
                ("orientation", ctypes.c_float * 3), ("angular_velocity", ctypes.c_float * 3),
                ("density", ctypes.c_float), ("fuel_fraction", ctypes.c_float), ("flame_fraction", ctypes.c_float),
                ("smoke_fraction", ctypes.c_float), ("size", ctypes.c_float)]


class Emitter(ctypes.Structure):
    """vg_emitter: PclOpEmit's template, spread, rate and remainder."""
    _fields_ = [("tmpl", ParticleValues), ("spread", ParticleValues), ("emit_rate", ctypes.c_float),
                ("remainder", ctypes.c_float)]


JITTER_HOST_RAND, JITTER_HASH = 0, 1


class Config(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_uint), ("device", ctypes.c_int), ("stream", ctypes.c_void_p),
                ("velocity_technique", ctypes.c_int), ("numerics", ctypes.c_int), ("poisson_solver", ctypes.c_int),
                ("warm_start", ctypes.c_int), ("viscosity", ctypes.c_float), ("poisson_tolerance", ctypes.c_double),
                ("poisson_max_cycles", ctypes.c_int), ("cascade_steps", ctypes.c_int),
                ("enable_stretch", ctypes.c_int), ("enable_diffusion", ctypes.c_int),
                ("boundary_copy_odd_x", ctypes.c_int), ("use_fixed_grid", ctypes.c_int),
                ("fixed_grid", GridGeom)]


class StepStats(ctypes.Structure):
    _fields_ = [("grid", GridGeom), ("tree_depth", ctypes.c_int), ("poisson_cycles", ctypes.c_int),
                ("poisson_relres", ctypes.c_double), ("poisson_relres0", ctypes.c_double),
                ("ms_total", ctypes.c_float), ("ms_poisson", ctypes.c_float),
                ("kernels_launched", ctypes.c_uint), ("warm_start_used", ctypes.c_int)]


_lib = None

EXPORTS = [
    "vg_status_string", "vg_last_error", "vg_abi_version", "vg_config_default", "vg_create", "vg_destroy",
    "vg_set_config", "vg_step", "vg_step_evolve", "vg_step_advect", "vg_step_device", "vg_step_evolve_device", "vg_get_velocity_grid", "vg_get_velocity_grid_device",
    "vg_get_vector_potential", "vg_get_stats", "vg_advect", "vg_advect_device", "vg_define_shape",
    "vg_set_poisson_schedule", "vg_get_poisson_schedule", "vg_set_coarsest_fp64",
    "vg_bin_device", "vg_partition_device", "vg_direct_device", "vg_tree_device", "vg_splat_device", "vg_boundary_vecpot_device",
    "vg_sor_device", "vg_cascade_device", "vg_multigrid_device", "vg_downsample_device", "vg_upsample_device",
    "vg_jacobian_curl_device", "vg_stretch_device", "vg_pse_device", "vg_gather_advect_device", "vg_synchronize",
    "vg_evolve_device", "vg_direct_noalloc", "vg_wind_device", "vg_kill_age_device", "vg_heat_pse_device",
    "vg_density_grid_device", "vg_gradient_device", "vg_baroclinic_device", "vg_signed_distance_device",
    "vg_marching_cubes_device", "vg_collide_vortons_device", "vg_collide_tracers_device",
    "vg_remove_embedded_device", "vg_emit_device", "vg_emit_grid_device", "vg_direct_grid_device",
    "vg_net_create", "vg_net_destroy", "vg_net_last_error", "vg_net_param_count", "vg_net_set_params",
    "vg_net_get_params", "vg_net_save", "vg_net_load", "vg_net_guess_device", "vg_net_backward_device",
    "vg_net_adam_step", "vg_net_get_grads", "vg_net_get_output", "vg_net_get_activation", "vg_net_get_gradient",
    "vg_net_synchronize",
    "vg_net_to_bf16_device", "vg_set_network",
    "vg_batch_create", "vg_batch_destroy", "vg_batch_last_error", "vg_batch_add", "vg_batch_load_network",
    "vg_batch_configure", "vg_batch_calibrate", "vg_batch_step", "vg_batch_synchronize", "vg_batch_autotune",
    "vg_batch_outside", "vg_batch_context", "vg_batch_size", "vg_batch_graph_info", "vg_batch_set_solver",
    "vg_batch_solver_info", "vg_team_barrier_check",
]


def lib():
    """Load libvortegrid.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libvortegrid.so not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                              f"(expected {LIB_PATH})")
        L = ctypes.CDLL(LIB_PATH)
        L.vg_status_string.restype = ctypes.c_char_p
        L.vg_last_error.restype = ctypes.c_char_p
        L.vg_last_error.argtypes = [ctypes.c_void_p]
        L.vg_abi_version.restype = ctypes.c_uint
        for name in EXPORTS:
            f = getattr(L, name)
            if name not in ("vg_status_string", "vg_last_error", "vg_abi_version"):
                f.restype = ctypes.c_int
        L.vg_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)]
        L.vg_destroy.argtypes = [ctypes.c_void_p]
        L.vg_set_config.argtypes = [ctypes.c_void_p, ctypes.POINTER(Config)]
        L.vg_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_float, ctypes.c_uint]
        L.vg_step_evolve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_uint]
        L.vg_step_advect.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_uint, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t]
        L.vg_step_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_size_t, ctypes.c_void_p, ctypes.c_float, ctypes.c_uint]
        L.vg_step_evolve_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_size_t, ctypes.c_void_p, ctypes.c_float, ctypes.c_uint]
        L.vg_get_velocity_grid.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(GridGeom)]
        L.vg_get_velocity_grid_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                  ctypes.POINTER(GridGeom)]
        L.vg_get_vector_potential.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                              ctypes.POINTER(GridGeom)]
        L.vg_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(StepStats)]
        L.vg_synchronize.argtypes = [ctypes.c_void_p]
        L.vg_direct_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_void_p]
        L.vg_evolve_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_float]
        L.vg_heat_pse_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_size_t, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.vg_density_grid_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_size_t, ctypes.c_float, ctypes.c_void_p]
        L.vg_gradient_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p, ctypes.c_void_p]
        L.vg_baroclinic_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                           ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_int)]
        L.vg_signed_distance_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p,
                                                ctypes.c_float, ctypes.c_int, ctypes.c_void_p]
        L.vg_marching_cubes_device.argtypes = [ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_void_p,
                                               ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                               ctypes.POINTER(ctypes.c_size_t)]
        _v, _i, _s, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_float
        L.vg_collide_vortons_device.argtypes = [_v, _v, _i, _v, _v, _v, _v, _s, _f, _f, _v, _v]
        L.vg_collide_tracers_device.argtypes = [_v, _v, _i, _v, _v, _v, _s, _v]
        L.vg_remove_embedded_device.argtypes = [_v, _v, _i, _v, _v, _v, _v, _s, ctypes.POINTER(ctypes.c_size_t)]
        L.vg_direct_grid_device.argtypes = [_v, ctypes.POINTER(GridGeom), _v, _v, _s, _v, _v]
        L.vg_emit_device.argtypes = [_v, ctypes.POINTER(Emitter), _f, ctypes.c_uint, ctypes.POINTER(Particles)]
        L.vg_emit_grid_device.argtypes = [_v, ctypes.POINTER(GridGeom), ctypes.c_uint, _v, _v, _s, _i, ctypes.c_uint,
                                          ctypes.POINTER(Particles)]
        L.vg_wind_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                     ctypes.c_float, ctypes.c_float]
        L.vg_kill_age_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_size_t)]
        L.vg_advect.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_float]
        L.vg_advect_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_float]
        L.vg_define_shape.argtypes = [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.POINTER(GridGeom)]
        vp, G, sz, fl, i = ctypes.c_void_p, ctypes.POINTER(GridGeom), ctypes.c_size_t, ctypes.c_float, ctypes.c_int
        L.vg_bin_device.argtypes = [vp, G, vp, sz, vp, vp]
        L.vg_partition_device.argtypes = [vp, G, vp, sz, vp, vp]
        L.vg_set_poisson_schedule.argtypes = [vp, i, i]
        L.vg_set_coarsest_fp64.argtypes = [vp, i]
        L.vg_get_poisson_schedule.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.vg_direct_device.argtypes = [vp, i, vp, vp, sz, vp, sz, fl, fl, vp]
        L.vg_tree_device.argtypes = [vp, i, G, vp, vp, sz, vp, sz, fl, fl, vp, vp, sz, ctypes.POINTER(ctypes.c_size_t)]
        L.vg_splat_device.argtypes = [vp, G, vp, vp, sz, fl, vp]
        L.vg_boundary_vecpot_device.argtypes = [vp, G, vp, vp, sz, i, vp]
        L.vg_sor_device.argtypes = [vp, G, vp, vp, i]
        L.vg_cascade_device.argtypes = [vp, G, vp, vp, i]
        L.vg_multigrid_device.argtypes = [vp, G, vp, vp, ctypes.c_double, i, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.vg_downsample_device.argtypes = [vp, G, vp, G, i, vp]
        L.vg_upsample_device.argtypes = [vp, G, vp, G, i, vp]
        L.vg_jacobian_curl_device.argtypes = [vp, G, vp, vp, vp]
        L.vg_stretch_device.argtypes = [vp, G, vp, vp, vp, sz, fl]
        L.vg_pse_device.argtypes = [vp, G, vp, vp, sz, fl, fl]
        L.vg_gather_advect_device.argtypes = [vp, G, vp, vp, vp, sz, fl]
        fp = ctypes.POINTER(ctypes.c_float)
        L.vg_net_create.argtypes = [i, vp, ctypes.c_uint, ctypes.POINTER(ctypes.c_void_p)]
        L.vg_net_destroy.argtypes = [vp]
        L.vg_net_last_error.argtypes = [vp]
        L.vg_net_last_error.restype = ctypes.c_char_p
        L.vg_net_param_count.restype = sz
        L.vg_net_set_params.argtypes = [vp, vp, sz, fl]
        L.vg_net_get_params.argtypes = [vp, vp, sz, fp]
        L.vg_net_save.argtypes = [vp, ctypes.c_char_p]
        L.vg_net_load.argtypes = [vp, ctypes.c_char_p]
        L.vg_net_guess_device.argtypes = [vp, G, vp, vp]
        L.vg_net_backward_device.argtypes = [vp, G, i, vp, vp, i, fp]
        L.vg_net_adam_step.argtypes = [vp, fl, fl, fl, fl]
        L.vg_net_get_grads.argtypes = [vp, vp, sz]
        L.vg_net_get_output.argtypes = [vp, vp, sz]
        L.vg_net_get_activation.argtypes = [vp, i, vp, sz]
        L.vg_net_get_gradient.argtypes = [vp, i, i, vp, sz]
        L.vg_net_synchronize.argtypes = [vp]
        L.vg_net_to_bf16_device.argtypes = [vp, vp, sz, vp]
        L.vg_set_network.argtypes = [vp, vp]
        ip = ctypes.POINTER(ctypes.c_int)
        L.vg_batch_create.argtypes = [i, i, ctypes.POINTER(ctypes.c_void_p)]
        L.vg_batch_destroy.argtypes = [vp]
        L.vg_batch_last_error.argtypes = [vp]
        L.vg_batch_last_error.restype = ctypes.c_char_p
        L.vg_batch_add.argtypes = [vp, ctypes.POINTER(Config), vp, vp, vp, sz, ip]
        L.vg_batch_load_network.argtypes = [vp, ctypes.c_char_p]
        L.vg_batch_configure.argtypes = [vp, i, i]
        L.vg_batch_calibrate.argtypes = [vp, fl]
        L.vg_batch_step.argtypes = [vp, fl, i]
        L.vg_batch_synchronize.argtypes = [vp]
        L.vg_batch_autotune.argtypes = [vp, fl, i, ip, i, ip, ip, fp]
        L.vg_batch_outside.argtypes = [vp, i, ip]
        L.vg_batch_context.argtypes = [vp, i]
        L.vg_batch_context.restype = vp
        L.vg_batch_size.argtypes = [vp]
        L.vg_batch_graph_info.argtypes = [vp, ip, ctypes.POINTER(sz), ctypes.POINTER(sz)]
        L.vg_batch_set_solver.argtypes = [vp, i, i, sz]
        L.vg_batch_solver_info.argtypes = [vp, ip, ip, ip, ip]
        L.vg_team_barrier_check.argtypes = [i, i, i, fl, ip, ip]
        if L.vg_abi_version() != 2:
            raise ImportError("libvortegrid ABI version mismatch")
        _lib = L
    return _lib


def default_config(**kw):
    cfg = Config()
    lib().vg_config_default(ctypes.byref(cfg))
    for k, v in kw.items():
        if k == "fixed_grid":
            cfg.fixed_grid = v
            cfg.use_fixed_grid = 1
        else:
            setattr(cfg, k, v)
    return cfg


class Context:
    """One vg_ctx: a VortonSim instance on one device and stream."""

    def __init__(self, cfg=None, **kw):
        self.cfg = cfg if cfg is not None else default_config(**kw)
        h = ctypes.c_void_p()
        st = lib().vg_create(ctypes.byref(self.cfg), ctypes.byref(h))
        if st != OK:
            raise VgError(st, "vg_create: " + lib().vg_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().vg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what):
        if st != OK:
            raise VgError(st, f"{what}: {lib().vg_last_error(self.h).decode()}")
        return st

    def set_config(self, **kw):
        for k, v in kw.items():
            if k == "fixed_grid":
                self.cfg.fixed_grid = v
                self.cfg.use_fixed_grid = 1
            else:
                setattr(self.cfg, k, v)
        self.check(lib().vg_set_config(self.h, ctypes.byref(self.cfg)), "vg_set_config")

    def synchronize(self):
        """Wait for the stream; raise for errors flagged by device stages."""
        self.check(lib().vg_synchronize(self.h), "vg_synchronize")

    def set_poisson_schedule(self, fp32_cycles=0, refinement_cycles=0):
        """Fixed multigrid schedule (no host round trip); (0, 0) = adaptive."""
        self.check(lib().vg_set_poisson_schedule(self.h, fp32_cycles, refinement_cycles), "vg_set_poisson_schedule")

    def set_coarsest_fp64(self, on=True):
        """Solve the multigrid's coarsest level in FP64 (True) or FP32 (False, the default)."""
        self.check(lib().vg_set_coarsest_fp64(self.h, int(bool(on))), "vg_set_coarsest_fp64")

    def poisson_schedule(self):
        """(FP32 cycles, refinement cycles) the last adaptive solve used."""
        k1, k2 = ctypes.c_int(), ctypes.c_int()
        self.check(lib().vg_get_poisson_schedule(self.h, ctypes.byref(k1), ctypes.byref(k2)),
                   "vg_get_poisson_schedule")
        return k1.value, k2.value

    def stats(self):
        s = StepStats()
        self.check(lib().vg_get_stats(self.h, ctypes.byref(s)), "vg_get_stats")
        return s


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


class VortonSim(Context):
    """VortonSim (VortonFluid/vortonSim.h:279-455) on the GPU."""

    def __init__(self, viscosity=0.01, cfg=None, **kw):
        if cfg is not None:
            super().__init__(cfg)
        else:
            super().__init__(viscosity=viscosity, **kw)

    def Update(self, particles, timeStep, uFrame=0, extra_min=None, extra_max=None):
        """FindBoundingBox + UpdateBoundingBox(final) + Update on host Particle records."""
        if particles.dtype.itemsize < 56 or not particles.flags.c_contiguous:
            raise ValueError("particles must be a C-contiguous array of Particle records")
        emin = np.ascontiguousarray(extra_min, np.float32) if extra_min is not None else None
        emax = np.ascontiguousarray(extra_max, np.float32) if extra_max is not None else None
        self.check(lib().vg_step(self.h, _ptr(particles), len(particles), particles.dtype.itemsize, _ptr(emin),
                                 _ptr(emax), timeStep, uFrame), "vg_step")

    def UpdateAndEvolve(self, particles, timeStep, uFrame=0, extra_min=None, extra_max=None):
        """Update followed by PclOpEvolve on the same host Particle records (vg_step_evolve)."""
        if particles.dtype.itemsize < 56 or not particles.flags.c_contiguous:
            raise ValueError("particles must be a C-contiguous array of Particle records")
        emin = np.ascontiguousarray(extra_min, np.float32) if extra_min is not None else None
        emax = np.ascontiguousarray(extra_max, np.float32) if extra_max is not None else None
        self.check(lib().vg_step_evolve(self.h, _ptr(particles), len(particles), particles.dtype.itemsize,
                                        _ptr(emin), _ptr(emax), timeStep, uFrame), "vg_step_evolve")

    def UpdateAndAdvect(self, particles, tracers, timeStep, uFrame=0, evolve=True, extra_min=None, extra_max=None):
        """One frame of both groups (vg_step_advect): Update (+ Evolve) on the vorton records, then
        AssignVelocityFromField (gain 1) + Evolve on the tracer records through the new velocity grid."""
        for a in (particles, tracers):
            if not a.flags.c_contiguous:
                raise ValueError("particle records must be C-contiguous")
        if particles.dtype.itemsize < 56 or tracers.dtype.itemsize < 24:
            raise ValueError("vorton records of at least 56 bytes and tracer records of at least 24 bytes")
        emin = np.ascontiguousarray(extra_min, np.float32) if extra_min is not None else None
        emax = np.ascontiguousarray(extra_max, np.float32) if extra_max is not None else None
        self.check(lib().vg_step_advect(self.h, _ptr(particles), len(particles), particles.dtype.itemsize,
                                        _ptr(emin), _ptr(emax), timeStep, uFrame, int(bool(evolve)), _ptr(tracers),
                                        len(tracers), tracers.dtype.itemsize), "vg_step_advect")

    def UpdateAndEvolveDevice(self, pos_size, angvel, vel, timeStep, uFrame=0, extra_minmax=None):
        """UpdateDevice followed by EvolveDevice on the same vortons (vg_step_evolve_device)."""
        e = np.ascontiguousarray(extra_minmax, np.float32) if extra_minmax is not None else None
        self.check(lib().vg_step_evolve_device(self.h, _ptr(pos_size), _ptr(angvel), _ptr(vel), pos_size.shape[0],
                                               _ptr(e), timeStep, uFrame), "vg_step_evolve_device")

    def UpdateDevice(self, pos_size, angvel, vel, timeStep, uFrame=0, extra_minmax=None):
        e = np.ascontiguousarray(extra_minmax, np.float32) if extra_minmax is not None else None
        self.check(lib().vg_step_device(self.h, _ptr(pos_size), _ptr(angvel), _ptr(vel), pos_size.shape[0], _ptr(e),
                                        timeStep, uFrame), "vg_step_device")

    def GetVelocityGrid(self):
        g = GridGeom()
        self.check(lib().vg_get_velocity_grid(self.h, None, 0, ctypes.byref(g)), "vg_get_velocity_grid")
        out = np.zeros((g.capacity, 3), np.float32)
        self.check(lib().vg_get_velocity_grid(self.h, _ptr(out), g.capacity, ctypes.byref(g)), "vg_get_velocity_grid")
        return out, g

    def GetVectorPotential(self):
        g = GridGeom()
        self.check(lib().vg_get_vector_potential(self.h, None, 0, ctypes.byref(g)), "vg_get_vector_potential")
        out = np.zeros((g.capacity, 3), np.float32)
        self.check(lib().vg_get_vector_potential(self.h, _ptr(out), g.capacity, ctypes.byref(g)),
                   "vg_get_vector_potential")
        return out, g

    def Advect(self, particles, timeStep):
        """AssignVelocityFromField (gain 1) + Evolve for tracer records."""
        self.check(lib().vg_advect(self.h, _ptr(particles), len(particles), particles.dtype.itemsize, timeStep),
                   "vg_advect")

    def EvolveDevice(self, pos4, vel4, timeStep):
        """PclOpEvolve on device float4 positions and velocities."""
        self.check(lib().vg_evolve_device(self.h, _ptr(pos4), _ptr(vel4), pos4.shape[0], timeStep),
                   "vg_evolve_device")

    def AdvectDevice(self, pos4, vel4, timeStep):
        self.check(lib().vg_advect_device(self.h, _ptr(pos4), _ptr(vel4), pos4.shape[0], timeStep),
                   "vg_advect_device")


class PclOpVortonSim:
    """IParticleOperation wrapper (VortonFluid/pclOpVortonSim.h:46-71):
    Operate(particles, timeStep, uFrame) runs one VortonSim step on the
    particle group's records; mMinCorner / mMaxCorner (the tracers' box) may be
    set to extend the grid."""

    def __init__(self, viscosity=0.01, **kw):
        self.mVortonSim = VortonSim(viscosity, **kw)
        self.mMinCorner = None
        self.mMaxCorner = None

    def Operate(self, particles, timeStep, uFrame=0):
        self.mVortonSim.Update(particles, timeStep, uFrame, self.mMinCorner, self.mMaxCorner)


class PclOpAssignVelocityFromFieldAndEvolve:
    """PclOpAssignVelocityFromField (gain 1) followed by PclOpEvolve for tracers,
    reading the velocity grid of a VortonSim's last step."""

    def __init__(self, vorton_sim):
        self.mVortonSim = vorton_sim

    def Operate(self, particles, timeStep, uFrame=0):
        self.mVortonSim.Advect(particles, timeStep)


def make_particles(pos, angvel=None, size=None):
    """Particle records from positions (and vorton angular velocity = vorticity/2, size = diameter)."""
    n = len(pos)
    p = np.zeros(n, PARTICLE_DTYPE)
    p["position"] = pos
    if angvel is not None:
        p["angular_velocity"] = angvel
    if size is not None:
        p["size"] = size
    p["density"] = 1.0
    return p


def define_shape(n, vmin, vmax, pow2=True):
    g = GridGeom()
    st = lib().vg_define_shape(n, _ptr(np.ascontiguousarray(vmin, np.float32)),
                               _ptr(np.ascontiguousarray(vmax, np.float32)), int(pow2), ctypes.byref(g))
    if st != OK:
        raise VgError(st, "vg_define_shape")
    return g


class ParticleGroup:
    """Device-resident arrays of one particle group (vg_particles), sized for
    `capacity` particles: pos_size, vel4, angvel4 (float4), density (float),
    birth (int), and orient4 / fire4 when asked.  `count` particles are live."""

    def __init__(self, capacity, device="cuda", orientation=False, fire=False):
        import torch
        f4 = lambda: torch.zeros((capacity, 4), dtype=torch.float32, device=device)  # noqa: E731
        self.pos_size, self.vel4, self.angvel4 = f4(), f4(), f4()
        self.orient4 = f4() if orientation else None
        self.fire4 = f4() if fire else None
        self.density = torch.zeros(capacity, dtype=torch.float32, device=device)
        self.birth = torch.zeros(capacity, dtype=torch.int32, device=device)
        self.capacity = capacity
        self.count = 0

    def c_struct(self):
        return Particles(_ptr(self.pos_size), _ptr(self.vel4), _ptr(self.angvel4), _ptr(self.orient4),
                         _ptr(self.density), _ptr(self.fire4), _ptr(self.birth), self.count, self.capacity)


class PclOpEmit:
    """IParticleOperation PclOpEmit (Particles/Operation/pclOpEmit.h:16-34) on a
    device particle group: Operate(group, timeStep, uFrame) emits mEmitRate
    particles a second from mTemplate varied by mSpread (dicts of the
    vg_particle_values fields); Emit(ctx, group, grid, multiplier, vortons) is
    the static tracer seeding on a grid (vortons: None or (pos_size, density)
    device arrays)."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.mTemplate = {}
        self.mSpread = {}
        self.mEmitRate = 60.0
        self.mRemainder = 0.0

    @staticmethod
    def _values(d):
        v = ParticleValues()
        for k, x in d.items():
            if isinstance(getattr(v, k), float):
                setattr(v, k, float(x))
            else:
                getattr(v, k)[:] = [float(c) for c in x]
        return v

    def Operate(self, group, timeStep, uFrame=0):
        em = Emitter(self._values(self.mTemplate), self._values(self.mSpread), self.mEmitRate, self.mRemainder)
        ps = group.c_struct()
        self.ctx.check(lib().vg_emit_device(self.ctx.h, ctypes.byref(em), timeStep, uFrame, ctypes.byref(ps)),
                       "PclOpEmit::Operate")
        self.mRemainder = em.remainder
        group.count = ps.count

    @staticmethod
    def Emit(ctx, group, grid, multiplier, vortons=None, jitter=JITTER_HOST_RAND, seed=0):
        if vortons is not None and int(vortons[1].shape[0]) == 0:
            return  # no vortons: no density deviation anywhere, so the reference emits nothing
        ps = group.c_struct()
        vp, vd, nv = (_ptr(vortons[0]), _ptr(vortons[1]), int(vortons[1].shape[0])) if vortons is not None else (
            None, None, 0)
        try:
            ctx.check(lib().vg_emit_grid_device(ctx.h, ctypes.byref(grid), multiplier, vp, vd, nv, jitter, seed,
                                                ctypes.byref(ps)), "PclOpEmit::Emit")
        finally:
            group.count = ps.count
