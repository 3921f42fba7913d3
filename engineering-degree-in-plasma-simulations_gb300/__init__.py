"""GB300-native electrostatic PIC + DSMC step loop (host mirror over the C ABI).

Python mirror of the reference's ch4/v3 class surface (Misquic/Engineering-degree-in-Plasma-
Simulations): World, Species, PotentialSolver and MC_MEX_Ionization, with the same method
names where the reference has them.  Every call goes through include/pic_gb300.h into
lib/libpic_gb300.so (hand-written sm_103a kernels).  There is no CPU fallback: if the
library or a CUDA device is missing, construction raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libpic_gb300.so")

PIC_OK, PIC_ERR_ARG, PIC_ERR_CUDA, PIC_ERR_NOT_CONVERGED, PIC_ERR_CAPACITY, PIC_ERR_DEVICE = range(6)
SOLVER_RBSOR, SOLVER_PCG, SOLVER_LEARNED = 0, 1, 2
STOP_REL_RHS, STOP_ABS_RMS, STOP_REL_CHARGE = 0, 1, 2  # Poisson stopping rules (pic_solver_set_stop)
WARM_PREVIOUS, WARM_EXTRAPOLATE = 0, 1  # start of a warm solve (pic_solver_set_warm_start)
GS, PCG = SOLVER_RBSOR, SOLVER_PCG  # reference SolverType names (PotentialSolver.h:24)

# ch4/v3/src/all.h:16-25
EPS0 = 8.85418782e-12
QE = 1.602176565e-19
AMU = 1.660538921e-27
ME = 9.10938215e-31
KB = 1.380648e-23

PARTICLE = np.dtype([("pos", "<f8", 3), ("vel", "<f8", 3), ("w", "<f8"), ("id", "<u8")])


class PicError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def build():
    from . import build as _b  # noqa: F401  (package-relative build recipe)

    return _b.build()


def library():
    """Load the CUDA library (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    import importlib

    importlib.import_module(__name__ + ".build").build()  # incremental: rebuilds only stale objects
    L = C.CDLL(LIB_PATH)
    vp, i, d, l, u64 = C.c_void_p, C.c_int, C.c_double, C.c_long, C.c_uint64
    pvp = C.POINTER(C.c_void_p)
    sig = {
        "pic_world_create": [pvp, i, i, i, vp, vp, i],
        "pic_world_destroy": [vp],
        "pic_world_set_time": [vp, d, i],
        "pic_world_advance_time": [vp, vp],
        "pic_world_get_ts": [vp, vp],
        "pic_world_get_time": [vp, vp],
        "pic_source_create": [vp, i, d, d, d, i, u64, vp],
        "pic_source_sample": [vp, i],
        "pic_autotune": [vp, vp, vp],
        "pic_launch_shapes": [vp, vp, vp, vp],
        "pic_set_launch_shapes": [vp, i, i, i],
        "pic_world_potential_energy": [vp, vp],
        "pic_species_sample_particles": [vp, i, l, vp, vp, vp],
        "pic_world_set_boundaries": [vp, vp, vp, vp],
        "pic_world_add_box": [vp, vp, vp, d],
        "pic_world_get_field": [vp, i, vp],
        "pic_world_set_field": [vp, i, vp],
        "pic_species_create": [vp, C.c_char_p, d, d, d, l, d, vp],
        "pic_species_add_particles": [vp, i, vp, vp, vp, vp, l, i],
        "pic_species_add_particles_batch": [vp, i, vp, vp, vp, vp, vp, vp, i, i],
        "pic_species_load_uniform": [vp, i, vp, vp, l, d, d, d, u64],
        "pic_species_count": [vp, i, vp],
        "pic_species_load_box_thermal": [vp, i, vp, vp, d, d, u64],
        "pic_species_get_particles": [vp, i, vp, vp, vp, vp, l, vp],
        "pic_species_push": [vp, i, d, i],
        "pic_species_number_density": [vp, i],
        "pic_species_get_den": [vp, i, vp],
        "pic_species_update_averages": [vp, i],
        "pic_species_get_den_avg": [vp, i, vp],
        "pic_species_sort": [vp, i, vp],
        "pic_species_sums": [vp, i, vp],
        "pic_charge_density": [vp],
        "pic_species_sample_moments": [vp, i],
        "pic_species_clear_samples": [vp, i],
        "pic_species_gas_properties": [vp, i, vp, vp],
        "pic_solver_configure": [vp, i, d, i, d],
        "pic_solver_solve": [vp, vp, vp],
        "pic_solver_compute_ef": [vp],
        "pic_solver_stats": [vp, vp, vp, vp],
        "pic_solver_set_stop": [vp, i, d],
        "pic_solver_set_warm_start": [vp, i],
        "pic_solver_set_warm_jacobi": [vp, i],
        "pic_solver_last_norms": [vp, vp],
        "pic_mcc_create": [vp, i, i, d, d, d, d, d, i, vp, vp, vp, i, u64],
        "pic_mcc_apply": [vp, d],
        "pic_mcc_stats": [vp, vp],
        "pic_dsmc_create": [vp, i, i, u64, vp],
        "pic_species_object_interaction": [vp, i, i, i, i, i, u64],
        "pic_species_object_stats": [vp, i, vp],
        "pic_dsmc_apply": [vp, i, d],
        "pic_dsmc_stats": [vp, i, vp, vp],
        "pic_loop_configure": [vp, i, i, vp, i, i, i],
        "pic_step": [vp],
        "pic_species_merge": [vp, i, i],
        "pic_merge_stats": [vp, vp],
        "pic_synchronize": [vp],
        "pic_debug_set_wait_polls": [vp, C.c_longlong],
        "pic_last_error": [C.c_char_p, i],
        "pic_timing_enable": [vp, i],
        "pic_timing_read": [vp, C.c_char_p, vp, vp],
        "pic_timing_reset": [vp],
        "pic_launch_count": [vp, vp],
        "pic_world_stream": [vp, pvp],
        "pic_number_density_noalloc": [i, i, i, vp, vp, vp, vp, vp, l, d, vp, vp],
        "pic_learned_levels": [vp, vp, vp, vp],
        "pic_world_set_slabs": [vp, i, vp, vp],
        "pic_mcc_set_slab_density": [vp, i, vp],
        "pic_learned_reset": [vp],
        "pic_learned_weights": [vp, vp, l, vp],
        "pic_learned_set_weights": [vp, vp, l],
        "pic_learned_apply": [vp, vp, vp],
        "pic_learned_loss_grad": [vp, vp, vp, vp, vp],
        "pic_learned_collect": [vp, i],
        "pic_learned_train": [vp, i, d, i, vp, vp, vp],
        "pic_learned_calibrate": [vp, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = L
    return L


def _check(rc, allow=()):
    if rc != PIC_OK and rc not in allow:
        buf = C.create_string_buffer(512)
        library().pic_last_error(buf, 512)
        raise PicError(rc, buf.value.decode(errors="replace"))
    return rc


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class World:
    """World(ni, nj, nk, x0, xm) -- ch4/v3/src/World.h:15-116 on one GPU."""

    def __init__(self, ni, nj, nk, x0, xm, device=0):
        self._L = library()
        h = C.c_void_p()
        _check(self._L.pic_world_create(C.byref(h), int(ni), int(nj), int(nk), _p(_f64(x0)), _p(_f64(xm)),
                                        int(device)))
        self._h = h
        self.ni, self.nj, self.nk = int(ni), int(nj), int(nk)
        self.nn = (self.ni, self.nj, self.nk)
        self.nv = self.ni * self.nj * self.nk
        self.num_cells = (self.ni - 1) * (self.nj - 1) * (self.nk - 1)
        self.x0 = np.asarray(x0, np.float64)
        self.xm = np.asarray(xm, np.float64)
        self.dx = (self.xm - self.x0) / (np.asarray(self.nn) - 1)
        self.species = []
        self.periodic = (0, 0, 0)

    def close(self):
        if getattr(self, "_h", None):
            self._L.pic_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # time (World.cpp:321-349)
    def setTime(self, dt, num_ts):
        _check(self._L.pic_world_set_time(self._h, float(dt), int(num_ts)))
        self.dt = float(dt)

    def advanceTime(self):
        r = C.c_int()
        _check(self._L.pic_world_advance_time(self._h, C.byref(r)))
        return bool(r.value)

    def getTs(self):
        t = C.c_int()
        _check(self._L.pic_world_get_ts(self._h, C.byref(t)))
        return t.value

    def getTime(self):
        """World::getTime (World.cpp:331-333): the sum of dt over the advanceTime calls."""
        t = C.c_double()
        _check(self._L.pic_world_get_time(self._h, C.byref(t)))
        return t.value

    def getPE(self):
        """World::getPE (World.cpp:108-119): 0.5 eps0 sum |E|^2 node_vol, summed on the device."""
        pe = C.c_double()
        _check(self._L.pic_world_potential_energy(self._h, C.byref(pe)))
        return pe.value

    def getDx(self):
        return self.dx.copy()

    def getCellVolume(self):
        return float(np.prod(self.dx))

    # boundaries
    def set_boundaries(self, periodic=(0, 0, 0), face_mode=(0,) * 6, face_phi=(0.0,) * 6):
        self.periodic = tuple(int(p) for p in periodic)
        _check(self._L.pic_world_set_boundaries(self._h, _p(np.asarray(periodic, np.int32)),
                                                _p(np.asarray(face_mode, np.int32)), _p(_f64(face_phi))))

    def set_slabs(self, phi_lo, phi_hi):
        """Stack independent instances along z: slab s has electrodes at phi_lo[s] (bottom plane) and
        phi_hi[s] (top plane); pass empty sequences for a single instance."""
        lo, hi = _f64(phi_lo), _f64(phi_hi)
        _check(self._L.pic_world_set_slabs(self._h, len(lo), _p(lo), _p(hi)))

    def dirichletBoundries(self, phi=0.0):
        """All walls Dirichlet at phi (World::dirichletBoundries, World.cpp:263-274)."""
        self.set_boundaries((0, 0, 0), (1,) * 6, (phi,) * 6)

    def addBox(self, center, sides, phi):
        """World::addObject<Rectangle>(pos, phi, sides) + computeObjectID."""
        _check(self._L.pic_world_add_box(self._h, _p(_f64(center)), _p(_f64(sides)), float(phi)))

    # fields
    def _get(self, which, comps=1):
        out = np.zeros(self.nv * comps)
        _check(self._L.pic_world_get_field(self._h, which, _p(out)))
        return out if comps == 1 else out.reshape(self.nv, comps)

    @property
    def phi(self):
        return self._get(0)

    @phi.setter
    def phi(self, v):
        _check(self._L.pic_world_set_field(self._h, 0, _p(_f64(v))))

    @property
    def rho(self):
        return self._get(1)

    @rho.setter
    def rho(self, v):
        _check(self._L.pic_world_set_field(self._h, 1, _p(_f64(v))))

    @property
    def node_vol(self):
        return self._get(2)

    @property
    def ef(self):
        return self._get(3, 3)

    @property
    def node_type(self):
        """World::node_type (World.h:17, 57): 0 REGULAR, 1 NEUMANN, 2 DIRICHLET."""
        return self._get(4).astype(np.int32)

    @property
    def object_id(self):
        """World::object_id (World.h:55): 1 on nodes inside a box, else 0."""
        return self._get(5).astype(np.int32)

    @ef.setter
    def ef(self, v):
        _check(self._L.pic_world_set_field(self._h, 3, _p(_f64(v))))

    def computeChargeDensity(self, species=None):
        """World::computeChargeDensity (World.cpp:193-200): den_s and rho = sum q_s den_s."""
        _check(self._L.pic_charge_density(self._h))

    # loop (main.cpp:177-286)
    def configure_loop(self, solve_each_step=True, sort_every=20, subcycle=(1, 1, 1, 1), merge_every=0,
                       merge_after=0, merge_min=10):
        _check(self._L.pic_loop_configure(self._h, int(solve_each_step), int(sort_every),
                                          _p(np.asarray(list(subcycle) + [1] * (4 - len(subcycle)), np.int32)),
                                          int(merge_every), int(merge_after), int(merge_min)))

    def autotune(self):
        """Measure launch shapes on this world's data and keep the fastest (pic_autotune)."""
        a, b = C.c_int(), C.c_int()
        _check(self._L.pic_autotune(self._h, C.byref(a), C.byref(b)))
        return self.launch_shapes()

    def launch_shapes(self):
        """Launch shapes in use: push CTAs per SM, CTAs of the streaming and of the CG stencil kernels."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(self._L.pic_launch_shapes(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return dict(push_ctas_per_sm=a.value, node_grid=b.value, cg_grid=c.value)

    def add_particles_batch(self, species, pos, vel, w, ids=None, rewind=True, sort=True):
        """Several species at once (pic_species_add_particles_batch): per species its (n, 3) positions
        and velocities and (n,) weights in FP64, as numpy arrays or as tensors in pinned host or
        device memory (objects with data_ptr(), read in place); with sort, each species leaves in
        cell order, its sort overlapping the next species' upload."""
        keep = []

        def addr(a, shape, dtype=np.float64):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                keep.append(a)
                return a.data_ptr()
            a = np.ascontiguousarray(a, dtype=dtype)
            if shape is not None:
                a = a.reshape(shape)
            keep.append(a)
            return a.ctypes.data

        k = len(species)
        sp = np.asarray([s.id for s in species], np.int32)
        ns = np.asarray([len(x) for x in w], np.int64)
        arr = lambda xs, shape: (C.c_void_p * k)(*[addr(x, shape) for x in xs])
        idp = None if ids is None else (C.c_void_p * k)(*[addr(x, None, np.uint64) for x in ids])
        _check(self._L.pic_species_add_particles_batch(self._h, k, _p(sp), arr(pos, (-1, 3)), arr(vel, (-1, 3)),
                                                       arr(w, (-1,)), idp, _p(ns), int(rewind), int(sort)))

    def set_launch_shapes(self, push_ctas_per_sm=0, node_grid=0, cg_grid=0):
        """Use launch shapes tuned on an earlier world of the same size (0: built-in default)."""
        _check(self._L.pic_set_launch_shapes(self._h, int(push_ctas_per_sm), int(node_grid), int(cg_grid)))

    def step(self):
        _check(self._L.pic_step(self._h))

    def synchronize(self):
        _check(self._L.pic_synchronize(self._h))

    # measurement
    def timing(self, on=True):
        _check(self._L.pic_timing_enable(self._h, int(on)))

    def timer(self, name):
        ms, n = C.c_double(), C.c_long()
        _check(self._L.pic_timing_read(self._h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def timing_reset(self):
        _check(self._L.pic_timing_reset(self._h))

    def launches(self):
        n = C.c_long()
        _check(self._L.pic_launch_count(self._h, C.byref(n)))
        return n.value


class Species:
    """Species(name, mass, charge, world, mpw0) -- ch4/v3/src/Species.h:31-133, particles on the GPU."""

    def __init__(self, name, mass, charge, world, mpw0, capacity=1 << 20, weight_bound=0.0):
        self.world = world
        self.name, self.mass, self.charge, self.mpw0 = name, float(mass), float(charge), float(mpw0)
        self.capacity = int(capacity)
        sid = C.c_int()
        _check(world._L.pic_species_create(world._h, name.encode(), self.mass, self.charge, self.mpw0,
                                           self.capacity, float(weight_bound), C.byref(sid)))
        self.id = sid.value
        world.species.append(self)

    @property
    def _L(self):
        return self.world._L

    def addParticles(self, pos, vel, w, ids=None, rewind=True):
        """Species::addParticle for arrays (Species.cpp:420-434)."""
        pos = _f64(pos, (-1, 3))
        vel = _f64(vel, (-1, 3))
        w = _f64(w, (-1,))
        idp = None if ids is None else np.ascontiguousarray(ids, np.uint64)
        _check(self._L.pic_species_add_particles(self.world._h, self.id, _p(pos), _p(vel), _p(w), _p(idp), len(w),
                                                 int(rewind)))

    def addParticle(self, pos, vel, macro_weight=None):
        self.addParticles([pos], [vel], [self.mpw0 if macro_weight is None else macro_weight])

    def loadUniform(self, lo, hi, n, T, w_mean=None, w_sigma=0.0, seed=1):
        _check(self._L.pic_species_load_uniform(self.world._h, self.id, _p(_f64(lo)), _p(_f64(hi)), int(n), float(T),
                                                float(self.mpw0 if w_mean is None else w_mean), float(w_sigma),
                                                int(seed)))

    def loadParticleBoxThermal(self, x0, sides, num_den, T, seed=1):
        """Species::loadParticleBoxThermal (Species.cpp:564-599), Philox draws."""
        _check(self._L.pic_species_load_box_thermal(self.world._h, self.id, _p(_f64(x0)), _p(_f64(sides)),
                                                    float(num_den), float(T), int(seed)))

    def getNumParticles(self):
        n = C.c_long()
        _check(self._L.pic_species_count(self.world._h, self.id, C.byref(n)))
        return n.value

    def getPartRef(self):
        """Host copy of the particles (Species::getPartRef, Species.cpp:823-825)."""
        n = self.getNumParticles()
        pos = np.zeros((max(n, 1), 3))
        vel = np.zeros((max(n, 1), 3))
        w = np.zeros(max(n, 1))
        ids = np.zeros(max(n, 1), np.uint64)
        got = C.c_long()
        _check(self._L.pic_species_get_particles(self.world._h, self.id, _p(pos), _p(vel), _p(w), _p(ids), max(n, 1),
                                                 C.byref(got)))
        n = got.value
        out = np.zeros(n, PARTICLE)
        out["pos"], out["vel"], out["w"], out["id"] = pos[:n], vel[:n], w[:n], ids[:n]
        return out

    def sample_particles(self, num_out):
        """(pos [m,3], vel [m,3]) of every (n // num_out)-th particle, the particle sample of
        Output::particlesOutput (Outputs.cpp:207-245); all particles when num_out > n."""
        pos = np.zeros((num_out, 3))
        vel = np.zeros((num_out, 3))
        got = C.c_long()
        _check(self._L.pic_species_sample_particles(self.world._h, self.id, int(num_out), _p(pos), _p(vel),
                                                    C.byref(got)))
        return pos[:got.value], vel[:got.value]

    def advance(self, dt, deposit=True):
        """One push with the species' current object interaction (see set_object_interaction)."""
        _check(self._L.pic_species_push(self.world._h, self.id, float(dt), int(deposit)))

    def set_object_interaction(self, mode, neutrals=None, spherium=None, sputtering=False, seed=None):
        """What a push does with particles that enter a box object: mode 0 removes them
        (Species::advanceElectrons), mode 1 is Species::advanceNonElectron(neutrals, spherium):
        neutral species bounce, ions are neutralised into `neutrals` (and sputter into
        `spherium` when `sputtering`).  pic_step pushes with the mode set here."""
        key = (int(mode), None if neutrals is None else neutrals.id, None if spherium is None else spherium.id,
               bool(sputtering), seed)
        if getattr(self, "_obj_key", None) == key:
            return
        seed = 0x0B1EC7 + 7919 * self.id if seed is None else int(seed)
        _check(self._L.pic_species_object_interaction(self.world._h, self.id, int(mode), key[1] if key[1] is not None
                                                      else -1, key[2] if key[2] is not None else -1,
                                                      int(bool(sputtering)), seed))
        self._obj_key = key

    def object_stats(self):
        out = np.zeros(4, np.uint64)
        _check(self._L.pic_species_object_stats(self.world._h, self.id, _p(out)))
        return dict(impacts=int(out[0]), bounces=int(out[1]), neutrals_created=int(out[2]),
                    sputtered_created=int(out[3]))

    def advanceElectrons(self, dt, deposit=True):  # Species.cpp:258-399: objects absorb
        self.set_object_interaction(0)
        self.advance(dt, deposit)

    def advanceNonElectron(self, neutrals, spherium, dt, deposit=True):  # Species.cpp:45-256
        sput = Config.getInstance().getSPUTTERING()
        self.set_object_interaction(1, neutrals, spherium, sput)
        self.advance(dt, deposit)

    def computeNumberDensity(self):
        _check(self._L.pic_species_number_density(self.world._h, self.id))

    @property
    def den(self):
        out = np.zeros(self.world.nv)
        _check(self._L.pic_species_get_den(self.world._h, self.id, _p(out)))
        return out

    @property
    def den_avg(self):
        out = np.zeros(self.world.nv)
        _check(self._L.pic_species_get_den_avg(self.world._h, self.id, _p(out)))
        return out

    def updateAverages(self):
        _check(self._L.pic_species_update_averages(self.world._h, self.id))

    def sortIndexes(self, counts=False):
        buf = np.zeros(self.world.num_cells, np.int32) if counts else None
        _check(self._L.pic_species_sort(self.world._h, self.id, _p(buf)))
        return buf

    def computeMacroParticlesCount(self):
        return self.sortIndexes(counts=True)

    def merge(self, min_count=10):
        _check(self._L.pic_species_merge(self.world._h, self.id, int(min_count)))

    def merge_stats(self):
        out = np.zeros(4, np.uint64)
        _check(self._L.pic_merge_stats(self.world._h, _p(out)))
        return dict(bins=int(out[0]), removed=int(out[1]), dropped=int(out[2]))

    def sampleMoments(self):
        _check(self._L.pic_species_sample_moments(self.world._h, self.id))

    def clearSamples(self):
        _check(self._L.pic_species_clear_samples(self.world._h, self.id))

    def computeGasProperties(self):
        """(vel [nv,3], T [nv]) as Species::computeGasProperties (Species.cpp:777-804)."""
        vel = np.zeros((self.world.nv, 3))
        T = np.zeros(self.world.nv)
        _check(self._L.pic_species_gas_properties(self.world._h, self.id, _p(vel), _p(T)))
        return vel, T

    def sums(self):
        out = np.zeros(5)
        _check(self._L.pic_species_sums(self.world._h, self.id, _p(out)))
        return out

    def getMicroCount(self):
        return self.sums()[0]

    def getMomentum(self):
        return self.sums()[1:4]

    def getKE(self):
        return self.sums()[4]


FACES = {"x-": 0, "x+": 1, "y-": 2, "y+": 3, "z-": 4, "z+": 5,
         "-x": 0, "+x": 1, "-y": 2, "+y": 3, "-z": 4, "+z": 5}  # inletName2Index, World.cpp:369-390


class ColdBeamSource:
    """ColdBeamSource(species, world, v_drift, den, inlet_face) -- ch4/v3/src/Source.h:42-52.

    Each step (pic_step, or sample()) injects (int)(den v_drift A dt / mpw0 + u) particles on the
    inlet face with velocity v_drift along the inward normal; the face becomes Dirichlet at 0 V."""

    T = 0.0

    def __init__(self, species, world, v_drift, den, inlet_face="-z", seed=1):
        face = FACES.get(str(inlet_face).lower())
        if face is None:
            raise ValueError("Passed wrong face name.")
        self.world = world
        sid = C.c_int()
        _check(world._L.pic_source_create(world._h, species.id, float(v_drift), float(den), float(self.T), face,
                                          int(seed), C.byref(sid)))
        self.id = sid.value

    def sample(self):
        _check(self.world._L.pic_source_sample(self.world._h, self.id))


class WarmBeamSource(ColdBeamSource):
    """WarmBeamSource(species, world, v_drift, den, T, inlet_face) -- ch4/v3/src/Source.h:55-66:
    the cold beam plus a Species::sampleV3th(T) thermal velocity."""

    def __init__(self, species, world, v_drift, den, T, inlet_face="-z", seed=1):
        self.T = float(T)
        super().__init__(species, world, v_drift, den, inlet_face, seed)


class PotentialSolver:
    """PotentialSolver(world, max_it, tol, type) -- ch4/v3/src/PotentialSolver.h:26-88.

    tol is the FP64 relative residual ||b - L phi|| / ||b|| of the reduced system, unless `stop`
    chooses another rule: STOP_ABS_RMS (the reference's sqrt(||r||^2 / nv) <= tol) or
    STOP_REL_CHARGE (relative to min(||b||, ||rho/eps0||))."""

    def __init__(self, world, max_solver_it, tolerance, solver_type=SOLVER_PCG, omega=1.4, stop=None):
        self.world = world
        _check(world._L.pic_solver_configure(world._h, int(solver_type), float(tolerance), int(max_solver_it),
                                             float(omega)))
        _check(world._L.pic_solver_set_stop(world._h, int(STOP_REL_RHS if stop is None else stop),
                                            float(tolerance)))
        self.iters, self.rel = 0, float("nan")

    def setWarmStart(self, mode):
        """WARM_PREVIOUS (the last potential) or WARM_EXTRAPOLATE (plus the last step's change)."""
        _check(self.world._L.pic_solver_set_warm_start(self.world._h, int(mode)))

    def setWarmJacobi(self, iterations):
        """Jacobi-PCG iterations a warm learned solve runs before the learned preconditioner."""
        _check(self.world._L.pic_solver_set_warm_jacobi(self.world._h, int(iterations)))

    def norms(self):
        """(||b - L phi||, ||b||, ||rho/eps0||) of the last solve's final residual (FREE nodes)."""
        out = np.zeros(3)
        _check(self.world._L.pic_solver_last_norms(self.world._h, _p(out)))
        return dict(r=out[0], b=out[1], charge=out[2])

    def solve(self, raise_on_fail=False):
        it, rel = C.c_int(), C.c_double()
        rc = _check(self.world._L.pic_solver_solve(self.world._h, C.byref(it), C.byref(rel)),
                    allow=() if raise_on_fail else (PIC_ERR_NOT_CONVERGED,))
        self.iters, self.rel = it.value, rel.value
        return rc == PIC_OK

    def computeEF(self):
        _check(self.world._L.pic_solver_compute_ef(self.world._h))

    def stats(self):
        a, b, c = C.c_long(), C.c_long(), C.c_long()
        _check(self.world._L.pic_solver_stats(self.world._h, C.byref(a), C.byref(b), C.byref(c)))
        return dict(solves=a.value, refinements=b.value, inner=c.value)


class LearnedPreconditioner:
    """The world's learned multilevel Poisson preconditioner (used by SOLVER_LEARNED)."""

    def __init__(self, world):
        self.world = world

    def levels(self):
        n = C.c_int()
        dims = np.zeros(36, np.int32)
        diag = np.zeros(12)
        _check(self.world._L.pic_learned_levels(self.world._h, C.byref(n), _p(dims), _p(diag)))
        return [tuple(dims[3 * k:3 * k + 3]) for k in range(n.value)], diag[:n.value].copy()

    def reset(self):
        _check(self.world._L.pic_learned_reset(self.world._h))

    def weights(self):
        n = C.c_long()
        _check(self.world._L.pic_learned_weights(self.world._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        _check(self.world._L.pic_learned_weights(self.world._h, _p(out), n.value, C.byref(n)))
        return out

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _check(self.world._L.pic_learned_set_weights(self.world._h, _p(w), w.size))

    def loss_grad(self, r, x):
        """Energy-norm loss of the pair (r, x) and its gradient (parameter layout), no update."""
        r, x = _f64(r).ravel(), _f64(x).ravel()
        loss = C.c_double()
        g = np.zeros(self.weights().size, np.float32)
        _check(self.world._L.pic_learned_loss_grad(self.world._h, _p(r), _p(x), C.byref(loss), _p(g)))
        return loss.value, g

    def collect(self, on=True):
        _check(self.world._L.pic_learned_collect(self.world._h, int(on)))

    def train(self, steps, lr=3e-3, pair_every=2):
        """One training round; returns (mean loss, validation iterations before, after, accepted)."""
        loss = C.c_double()
        it = np.zeros(2, np.int32)
        acc = C.c_int()
        _check(self.world._L.pic_learned_train(self.world._h, int(steps), float(lr), int(pair_every), C.byref(loss),
                                               _p(it), C.byref(acc)))
        return loss.value, int(it[0]), int(it[1]), bool(acc.value)

    def calibrate(self):
        """Level gains judged by validation solves (pic_learned_calibrate); returns (before, after)."""
        it = np.zeros(2, np.int32)
        _check(self.world._L.pic_learned_calibrate(self.world._h, _p(it)))
        return int(it[0]), int(it[1])

    def apply(self, r):
        """z = B r over all nodes (r read on FREE nodes; z zero elsewhere)."""
        r = _f64(r).ravel()
        z = np.zeros_like(r)
        _check(self.world._L.pic_learned_apply(self.world._h, _p(r), _p(z)))
        return z


class Config:
    """The reference's Config singleton (ch4/v3/src/Config.h), for the switch the pushes read."""

    _instance = None

    def __init__(self):
        self._sputtering = False

    @classmethod
    def getInstance(cls):
        if cls._instance is None:
            cls._instance = cls()
        return cls._instance

    def getSPUTTERING(self):
        return self._sputtering

    def setSPUTTERING(self, on):
        self._sputtering = bool(on)


class MC_MEX_Ionization:
    """Electron-impact ionisation / elastic collisions against a background gas
    (GPU form of ch4/v3/src/Interactions.h:98-143)."""

    def __init__(self, electrons, ions, world, n_neutral, T_neutral, m_neutral, E_ion_eV, table_E, table_s,
                 sigma_ion_kind=0, sigma_ion_params=(1.015e-18, 9.793, 61.81, 0.0), B_inc=10.0, seed=12345):
        self.world = world
        self._tE = _f64(table_E)
        self._tS = _f64(table_s)
        _check(world._L.pic_mcc_create(world._h, electrons.id, ions.id, float(n_neutral), float(T_neutral),
                                       float(m_neutral), float(E_ion_eV), float(B_inc), int(sigma_ion_kind),
                                       _p(_f64(list(sigma_ion_params) + [0.0] * (4 - len(sigma_ion_params)))),
                                       _p(self._tE), _p(self._tS), len(self._tE), int(seed)))

    def apply(self, dt):
        _check(self.world._L.pic_mcc_apply(self.world._h, float(dt)))

    def set_slab_density(self, n_neutral):
        """Background density of every instance slab."""
        n = _f64(n_neutral)
        _check(self.world._L.pic_mcc_set_slab_density(self.world._h, len(n), _p(n)))

    def stats(self):
        out = np.zeros(4, np.uint64)
        _check(self.world._L.pic_mcc_stats(self.world._h, _p(out)))
        return dict(candidates=int(out[0]), collisions=int(out[1]), ionizations=int(out[2]), lost=int(out[3]))


class DSMC_MEX:
    """VHS particle-particle collisions of one species with itself, DSMC_MEX(species, world), or
    between two species of equal mpw0, DSMC_MEX(species1, species2, world)
    (ch4/v3/src/Interactions.h:42-66).  World.step() applies it every step before the pushes."""

    def __init__(self, species1, species2_or_world, world=None, seed=12345):
        if world is None:
            species2, world = None, species2_or_world
        else:
            species2 = species2_or_world
        self.world = world
        i = C.c_int(0)
        _check(world._L.pic_dsmc_create(world._h, species1.id, -1 if species2 is None else species2.id, int(seed),
                                        C.byref(i)))
        self.id = i.value

    def apply(self, dt):
        _check(self.world._L.pic_dsmc_apply(self.world._h, self.id, float(dt)))

    def stats(self):
        out = np.zeros(2, np.uint64)
        sv = C.c_double(0)
        _check(self.world._L.pic_dsmc_stats(self.world._h, self.id, _p(out), C.byref(sv)))
        return dict(collisions=int(out[0]), pairs=int(out[1]), sigma_v_rel_max=sv.value)
