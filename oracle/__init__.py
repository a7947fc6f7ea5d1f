"""CPU oracle for the VortonSim velocity-from-vorticity step.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg (``cpu_baseline`` and ``--impl reference``)
may import this package, and only as the checker or the timed CPU baseline.
The product package ``vortegrid_gb300`` never imports it.

Two libraries are wrapped:
  * ``liboracle`` -- ``vg_oracle.c``, a plain-C restatement of the reference's
    algorithms (each function cites the reference file:line it follows) plus
    the strict FP64 direct-sum oracle.  Built by ``build()`` below.
  * ``libvgref_{serial,mt}`` -- the reference's own C++ (staged by
    ``ref_build/prepare.py`` and built by ``ref_build/Makefile``), used to pin
    the restatement and as the CPU baseline.  Optional: absent when neither the
    reference tree nor a staged copy of it is available.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# Location of a VorteGrid checkout to stage the reference build from (no default:
# hosts without it use an already staged copy in _ref/src, or the C oracle alone).
REF_TREE = os.environ.get("VG_REFERENCE_TREE", "")


def build(quiet=True):
    """Compile vg_oracle.c (and, when reference sources are staged, the
    reference harness) for this host."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "vg_oracle.c")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "vg_oracle.h"))):
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off",
                               "-o", LIB, src, "-lm"])
    staged = os.path.join(REF_DIR, "src", ".staged")
    if not os.path.exists(staged) and REF_TREE and os.path.isdir(REF_TREE):
        subprocess.check_call(["python3", os.path.join(HERE, "ref_build", "prepare.py"), REF_TREE],
                              stdout=subprocess.DEVNULL if quiet else None)
    if os.path.exists(staged):
        # The reference build is optional (it pins goldens here and is the CPU
        # baseline); a host where it does not build falls back to the C oracle.
        log = os.path.join(REF_DIR, "build.log")
        with open(log, "w") as fh:
            r = subprocess.run(["make", "-C", os.path.join(HERE, "ref_build"), "-j8"], stdout=fh,
                               stderr=subprocess.STDOUT)
        if r.returncode != 0 and not quiet:
            print(f"oracle: the reference's own code did not build on this host (see {log})")


class Geom(ctypes.Structure):
    """vgo_geom: UniformGridGeometry fields."""
    _fields_ = [("mn", ctypes.c_float * 3), ("ext", ctypes.c_float * 3), ("cell", ctypes.c_float * 3),
                ("cpe", ctypes.c_float * 3), ("np", ctypes.c_uint * 3)]

    @property
    def points(self):
        return tuple(int(v) for v in self.np)

    @property
    def capacity(self):
        return int(self.np[0]) * int(self.np[1]) * int(self.np[2])

    def as12(self):
        return np.array(list(self.mn) + list(self.ext) + list(self.cell) + list(self.cpe), dtype=np.float32)

    @staticmethod
    def from12(g12, np3):
        g = Geom()
        for a in range(3):
            g.mn[a] = float(g12[a]); g.ext[a] = float(g12[3 + a])
            g.cell[a] = float(g12[6 + a]); g.cpe[a] = float(g12[9 + a]); g.np[a] = int(np3[a])
        return g


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        _lib.vgo_finvsqrtf.restype = ctypes.c_float
        _lib.vgo_finvsqrtf.argtypes = [ctypes.c_float]
        _lib.vgo_influence_tree.restype = ctypes.c_size_t
        _lib.vgo_offset_of_position.restype = ctypes.c_uint
        _lib.vgo_nested_shape.restype = ctypes.c_int
        _lib.vgo_relres_f64.restype = ctypes.c_double
        _lib.vgo_relres_f64d.restype = ctypes.c_double
        _lib.vgo_tree_interactions.restype = ctypes.c_size_t
        _lib.vgo_baroclinic.restype = ctypes.c_int
        _lib.vgo_marching_cubes.restype = ctypes.c_size_t
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def define_shape(n, vmin, vmax, pow2=True):
    g = Geom()
    lib().vgo_define_shape(ctypes.c_size_t(n), _p(f32(vmin)), _p(f32(vmax)), ctypes.c_int(int(pow2)), ctypes.byref(g))
    return g


def step_geometry(pos, radius, extra_min=None, extra_max=None):
    g = Geom()
    pos = f32(pos)
    lib().vgo_step_geometry(_p(pos), ctypes.c_size_t(len(pos)), ctypes.c_float(radius),
                            _p(f32(extra_min)) if extra_min is not None else None,
                            _p(f32(extra_max)) if extra_max is not None else None, ctypes.byref(g))
    return g


def indices_of_position(g, pos):
    pos = f32(pos)
    idx = np.zeros((len(pos), 3), np.uint32)
    off = np.zeros(len(pos), np.uint32)
    lib().vgo_indices_batch(ctypes.byref(g), _p(pos), ctypes.c_size_t(len(pos)), _p(idx), _p(off))
    return idx, off


def partition(g, pos):
    """PartitionParticles cell lists: (start[points + 2], items[n])."""
    pos = f32(pos)
    start = np.zeros(g.capacity + 2, np.uint32)
    items = np.zeros(max(len(pos), 1), np.uint32)
    lib().vgo_partition(ctypes.byref(g), _p(pos), ctypes.c_size_t(len(pos)), _p(start), _p(items))
    return start, items[: len(pos)]


def nested_shape(g):
    layers = (Geom * 32)()
    dec = np.zeros(96, np.uint32)
    depth = lib().vgo_nested_shape(ctypes.byref(g), layers, _p(dec))
    return [layers[i] for i in range(depth)], dec[:3 * depth].reshape(depth, 3)


def direct(kind, pos, angvel, size, q, spread_range=1.0, spread_circ=1.0, f64=False):
    pos, angvel, size, q = f32(pos), f32(angvel), f32(size), f32(q)
    out = np.zeros((len(q), 3), np.float64 if f64 else np.float32)
    fn = lib().vgo_direct_f64 if f64 else lib().vgo_direct
    fn(ctypes.c_int(kind), _p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), _p(q), ctypes.c_size_t(len(q)),
       ctypes.c_float(spread_range), ctypes.c_float(spread_circ), _p(out))
    return out


def influence_tree(pos, angvel, size, g):
    pos, angvel, size = f32(pos), f32(angvel), f32(size)
    total = lib().vgo_influence_tree(_p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g), None)
    out = np.zeros((total, 7), np.float32)
    lib().vgo_influence_tree(_p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g), _p(out))
    return out


def tree(kind, pos, angvel, size, g, q, spread_range=1.0, spread_circ=1.0):
    pos, angvel, size, q = f32(pos), f32(angvel), f32(size), f32(q)
    out = np.zeros((len(q), 3), np.float32)
    lib().vgo_tree(ctypes.c_int(kind), _p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g),
                   _p(q), ctypes.c_size_t(len(q)), ctypes.c_float(spread_range), ctypes.c_float(spread_circ), _p(out))
    return out


def tree_interactions(g, q):
    """Pair laws the treecode walk evaluates over the queries q."""
    q = f32(q)
    return int(lib().vgo_tree_interactions(ctypes.byref(g), _p(q), ctypes.c_size_t(len(q))))


def splat(pos, angvel, size, g, scale=-1.0):
    pos, angvel, size = f32(pos), f32(angvel), f32(size)
    out = np.zeros((g.capacity, 3), np.float32)
    lib().vgo_splat(_p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g), ctypes.c_float(scale),
                    _p(out))
    return out


def boundary_vecpot(pos, angvel, size, g, boundaries_only=True, copy_odd_x=True):
    pos, angvel, size = f32(pos), f32(angvel), f32(size)
    out = np.zeros((g.capacity, 3), np.float32)
    lib().vgo_boundary_vecpot(_p(pos), _p(angvel), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g),
                              ctypes.c_int(int(boundaries_only)), ctypes.c_int(int(copy_odd_x)), _p(out))
    return out


def sor(g, soln, lap, steps):
    s = f32(soln).copy()
    lib().vgo_sor(ctypes.byref(g), _p(s), _p(f32(lap)), ctypes.c_int(steps))
    return s


def downsample(fine, fv, coarse, inject=True):
    out = np.zeros((coarse.capacity, 3), np.float32)
    lib().vgo_downsample(ctypes.byref(fine), _p(f32(fv)), ctypes.c_int(int(inject)), ctypes.byref(coarse), _p(out))
    return out


def upsample(coarse, cv, fine, fine_init, interior_only=True):
    out = f32(fine_init).copy()
    lib().vgo_upsample(ctypes.byref(coarse), _p(f32(cv)), ctypes.byref(fine), ctypes.c_int(int(interior_only)),
                       _p(out))
    return out


def cascade(g, soln, rhs, steps=16):
    s = f32(soln).copy()
    lib().vgo_cascade(ctypes.byref(g), _p(s), _p(f32(rhs)), ctypes.c_int(steps))
    return s


def jacobian(g, vec):
    out = np.zeros((g.capacity, 9), np.float32)
    lib().vgo_jacobian(ctypes.byref(g), _p(f32(vec)), _p(out))
    return out


def curl_from_jacobian(jac):
    jac = f32(jac)
    out = np.zeros((len(jac), 3), np.float32)
    lib().vgo_curl_from_jacobian(ctypes.c_size_t(len(jac)), _p(jac), _p(out))
    return out


def stretch(pos, angvel, g, jac9, dt):
    w = f32(angvel).copy()
    pos = f32(pos)
    lib().vgo_stretch(_p(pos), _p(w), ctypes.c_size_t(len(pos)), ctypes.byref(g), _p(f32(jac9)), ctypes.c_float(dt))
    return w


def pse(pos, angvel, size, g, viscosity, dt, symmetric=False):
    w = f32(angvel).copy()
    pos, size = f32(pos), f32(size)
    fn = lib().vgo_pse_symmetric if symmetric else lib().vgo_pse_sequential
    fn(_p(pos), _p(w), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g), ctypes.c_float(viscosity),
       ctypes.c_float(dt))
    return w


def gather(g, velgrid, pos):
    pos = f32(pos)
    out = np.zeros((len(pos), 3), np.float32)
    lib().vgo_gather(ctypes.byref(g), _p(f32(velgrid)), _p(pos), ctypes.c_size_t(len(pos)), _p(out))
    return out


def evolve(pos, vel, dt):
    p = f32(pos).copy()
    lib().vgo_evolve(_p(p), _p(f32(vel)), ctypes.c_size_t(len(p)), ctypes.c_float(dt))
    return p


def heat_pse(pos, density, size, g, diffusivity, ambient, dt, symmetric=False):
    d = np.ascontiguousarray(density, np.float32).copy()
    fn = lib().vgo_heat_pse_symmetric if symmetric else lib().vgo_heat_pse_sequential
    fn(_p(f32(pos)), _p(d), _p(f32(size)), ctypes.c_size_t(len(d)), ctypes.byref(g), ctypes.c_float(diffusivity),
       ctypes.c_float(ambient), ctypes.c_float(dt))
    return d


def density_grid(pos, size, density, g, ambient):
    """PopulateDensityAndMassFractionGrids (density): float32[points]."""
    out = np.zeros(g.capacity, np.float32)
    d = np.ascontiguousarray(density, np.float32)
    lib().vgo_density_grid(_p(f32(pos)), _p(f32(size)), _p(d), ctypes.c_size_t(len(d)), ctypes.byref(g),
                           ctypes.c_float(ambient), _p(out))
    return out


def gradient(g, v):
    """ComputeGradient of a scalar grid: float32[points, 3]."""
    out = np.zeros((g.capacity, 3), np.float32)
    lib().vgo_gradient(ctypes.byref(g), _p(np.ascontiguousarray(v, np.float32)), _p(out))
    return out


def baroclinic(pos, angvel, size, density, g, grav, ambient, dt):
    """Baroclinic generation on the density-grid path: (applied, new angvel)."""
    w = f32(angvel).copy()
    d = np.ascontiguousarray(density, np.float32)
    r = lib().vgo_baroclinic(_p(f32(pos)), _p(w), _p(f32(size)), _p(d), ctypes.c_size_t(len(d)), ctypes.byref(g),
                             _p(f32(grav)), ctypes.c_float(ambient), ctypes.c_float(dt))
    return bool(r), w


def signed_distance(g, density, ambient, sumstats=0):
    """PopulateSignedDistanceGridFromDensityGrid: float32[points] (NaN where unreached).
    sumstats 0: the reference's float sums for the density statistics; 1: double sums."""
    out = np.zeros(g.capacity, np.float32)
    lib().vgo_signed_distance(ctypes.byref(g), _p(np.ascontiguousarray(density, np.float32)), ctypes.c_float(ambient),
                              ctypes.c_int(sumstats), _p(out))
    return out


def marching_cubes(g, v, iso):
    """Isosurface triangles: (positions float32[t, 3, 3], normals float32[t, 3, 3])."""
    v = np.ascontiguousarray(v, np.float32)
    n = lib().vgo_marching_cubes(ctypes.byref(g), _p(v), ctypes.c_float(iso), None, None, ctypes.c_size_t(0))
    verts = np.zeros((max(n, 1), 3, 3), np.float32)
    norms = np.zeros((max(n, 1), 3, 3), np.float32)
    lib().vgo_marching_cubes(ctypes.byref(g), _p(v), ctypes.c_float(iso), _p(verts), _p(norms), ctypes.c_size_t(n))
    return verts[:n], norms[:n]


def marching_cubes_table():
    cnt = np.zeros(256, np.int32)
    tri = np.zeros((256, 15), np.int32)
    lib().vgo_marching_cubes_table(_p(cnt), _p(tri))
    return cnt, tri


def body(shape, position, dims, hole=False, velocity=(0, 0, 0), angular_velocity=(0, 0, 0), orientation=None,
         temperature=300.0, conductivity=0.0):
    """One rigid body as 32 floats (shape 0 sphere with radius dims[0], 1 box of dims)."""
    b = np.zeros(32, np.float32)
    b[0] = shape
    b[1] = 1.0 if hole else 0.0
    b[2:5], b[5:8], b[8:11] = position, velocity, angular_velocity
    b[11:20] = np.asarray(np.eye(3) if orientation is None else orientation, np.float32).ravel()
    d = np.atleast_1d(np.asarray(dims, np.float32))
    b[20:20 + len(d)] = d
    b[23], b[24] = temperature, conductivity
    return b


def collide_vortons(pos, vel, angvel, size, density, bodies, ambient=1.0, specific_heat=1.0):
    """CollideVortonsSlice per body: (pos, vel, angvel, density, per-body float32[nb, 9])."""
    p, v, w, d = f32(pos).copy(), f32(vel).copy(), f32(angvel).copy(), f32(density).copy()
    b = f32(bodies).reshape(-1, 32)
    out = np.zeros((len(b), 9), np.float32)
    lib().vgo_collide_vortons(_p(p), _p(v), _p(w), _p(f32(size)), _p(d), ctypes.c_size_t(len(p)), _p(b),
                              ctypes.c_int(len(b)), ctypes.c_float(ambient), ctypes.c_float(specific_heat), _p(out))
    return p, v, w, d, out


def collide_tracers(pos, vel, size, density, bodies):
    """CollideTracersSlice per body: (pos, vel, per-body float32[nb, 6])."""
    p, v = f32(pos).copy(), f32(vel).copy()
    b = f32(bodies).reshape(-1, 32)
    out = np.zeros((len(b), 6), np.float32)
    lib().vgo_collide_tracers(_p(p), _p(v), _p(f32(size)), _p(f32(density)), ctypes.c_size_t(len(p)), _p(b),
                              ctypes.c_int(len(b)), _p(out))
    return p, v, out


def remove_embedded(pos, size, bodies):
    """RemoveEmbeddedParticles: the survivors' original indices in the order left."""
    b = f32(bodies).reshape(-1, 32)
    order = np.zeros(max(len(pos), 1), np.uint32)
    m = ctypes.c_size_t()
    lib().vgo_remove_embedded(_p(f32(pos)), _p(f32(size)), ctypes.c_size_t(len(pos)), _p(b), ctypes.c_int(len(b)),
                              _p(order), ctypes.byref(m))
    return order[: m.value].copy()


def kill_age(birth, frame, age_max):
    """Survivors' original indices in the order PclOpKillAge leaves them."""
    b = np.ascontiguousarray(birth, np.int32)
    order = np.zeros(len(b), np.uint32)
    m = ctypes.c_size_t()
    lib().vgo_kill_age(_p(b), ctypes.c_size_t(len(b)), ctypes.c_uint(frame), ctypes.c_int(age_max), _p(order),
                       ctypes.byref(m))
    return order[: m.value].copy()


def wind(vel, wind_vec, wind_weight, src_weight):
    v = f32(vel).copy()
    lib().vgo_wind(_p(v), ctypes.c_size_t(len(v)), _p(f32(wind_vec)), ctypes.c_float(wind_weight),
                   ctypes.c_float(src_weight))
    return v


def relres(g, a, b):
    if a.dtype == np.float64:
        return lib().vgo_relres_f64d(ctypes.byref(g), _p(np.ascontiguousarray(a)), _p(f32(b)))
    return lib().vgo_relres_f64(ctypes.byref(g), _p(f32(a)), _p(f32(b)))


def step_fields(pos, vel, angvel, size, g, dt, viscosity, pse_mode=0):
    pos, size = f32(pos), f32(size)
    v = f32(vel).copy()
    w = f32(angvel).copy()
    vg = np.zeros((g.capacity, 3), np.float32)
    ap = np.zeros((g.capacity, 3), np.float32)
    nv = np.zeros((g.capacity, 3), np.float32)
    lib().vgo_step_fields(_p(pos), _p(v), _p(w), _p(size), ctypes.c_size_t(len(pos)), ctypes.byref(g),
                          ctypes.c_float(dt), ctypes.c_float(viscosity), ctypes.c_int(pse_mode), _p(vg), _p(ap), _p(nv))
    return v, w, vg, ap, nv


# ---------------------------------------------------------------- reference

def ref_available(kind="serial"):
    return os.path.exists(os.path.join(REF_DIR, f"libvgref_{kind}.so"))


_ref = {}


def ref(kind="serial"):
    """The reference's own code (serial: USE_TBB=0; mt: USE_TBB=1 on a
    std::thread TBB stand-in using NUMBER_OF_PROCESSORS threads)."""
    if kind not in _ref:
        path = os.path.join(REF_DIR, f"libvgref_{kind}.so")
        L = ctypes.CDLL(path)
        L.vgref_sizeof_particle.restype = ctypes.c_size_t
        L.vgref_influence_tree.restype = ctypes.c_size_t
        L.vgref_nested_grid_shape.restype = ctypes.c_int
        L.vgref_step.restype = ctypes.c_int
        _ref[kind] = L
    return _ref[kind]


def srand(seed):
    """Seed the C library's rand(), the draws the reference's emitters consume."""
    ctypes.CDLL(None).srand(ctypes.c_uint(seed))


def rand_max():
    return int(lib().vgo_rand_max())


def jitter_hash(seed, d):
    """Draw d of the device emitter's counter-based jitter stream."""
    f = lib().vgo_jitter_hash
    f.argtypes = [ctypes.c_uint, ctypes.c_uint64]
    return int(f(seed, d))


def emit_grid(g, multiplier, vortons=None, host_rand=True, seed=0):
    """PclOpEmit::Emit on grid g (vortons: None or (pos, density)); host_rand
    draws from the C library's rand() as it stands.  Returns (pos, density,
    size) of the particles emitted."""
    m = int(multiplier)
    cells = int(np.prod([int(v) - 1 for v in g.np]))
    cap = cells * m ** 3
    pos = np.zeros((max(cap, 1), 3), np.float32)
    dens = np.zeros(max(cap, 1), np.float32)
    size = np.zeros(max(cap, 1), np.float32)
    cnt = ctypes.c_size_t()
    vp, vd, nv = (f32(vortons[0]), f32(vortons[1]), len(vortons[1])) if vortons is not None else (
        np.zeros((1, 3), np.float32), np.zeros(1, np.float32), 0)
    lib().vgo_emit_grid(ctypes.byref(g), ctypes.c_uint(m), _p(vp), _p(vd), ctypes.c_size_t(nv),
                        ctypes.c_int(vortons is not None), ctypes.c_int(bool(host_rand)), ctypes.c_uint(seed),
                        _p(pos), _p(dens), _p(size), ctypes.c_size_t(cap), ctypes.byref(cnt))
    k = cnt.value
    return pos[:k].copy(), dens[:k].copy(), size[:k].copy()


def emit_operate(tmpl, spread, rate, dts, frame0=0, remainder=0.0, host_rand=True, seed=0):
    """PclOpEmit::Operate for each time step in dts (frames frame0, frame0 + 1,
    ...), appending to one array: (records float32[k, 18] -- 17 values and the
    birth frame -- and the remainder after each call)."""
    f = lib().vgo_emit_operate
    f.restype = ctypes.c_size_t
    t, s = f32(tmpl).ravel(), f32(spread).ravel()
    rem = ctypes.c_float(remainder)
    draw = ctypes.c_uint64(0)
    recs, rems = [], []
    for i, dt in enumerate(dts):
        cap = int(float(dt) * float(rate) + rem.value) + 2
        buf = np.zeros((cap, 18), np.float32)
        k = f(_p(t), _p(s), ctypes.c_float(rate), ctypes.byref(rem), ctypes.c_float(dt),
              ctypes.c_uint(frame0 + i), ctypes.c_int(bool(host_rand)), ctypes.c_uint(seed), ctypes.byref(draw),
              _p(buf), ctypes.c_size_t(cap))
        recs.append(buf[:k])
        rems.append(rem.value)
    return np.concatenate(recs) if recs else np.zeros((0, 18), np.float32), np.array(rems, np.float32)
