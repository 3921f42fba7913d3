"""ctypes bindings for the CPU oracles -- TEST INFRASTRUCTURE ONLY.

`Port` wraps oracle/_build/libpicoracle.so (the plain-C FP64 restatement in pic_oracle.c);
`Ref` wraps oracle/_ref/libpicref.so (the reference's own ch4/v3 classes compiled from
their sources with ref_harness.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module; the CUDA product path never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpicoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpicref.so")


def reference_root():
    """Location of the reference tree: PIC_REFERENCE_ROOT, else the build recipe's default."""
    root = os.environ.get("PIC_REFERENCE_ROOT")
    if root:
        return root
    try:
        out = subprocess.run(["make", "-s", "print-ref"], cwd=HERE, check=True, capture_output=True, text=True)
        return out.stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""


# physical constants of ch4/v3/src/all.h:16-25
EPS0 = 8.85418782e-12
QE = 1.602176565e-19
AMU = 1.660538921e-27
ME = 9.10938215e-31
KB = 1.380648e-23
PI_REF = 3.141592653

FREE, FIXED, MIRROR, ALIAS = 0, 1, 2, 3

PARTICLE = np.dtype([("pos", "<f8", 3), ("vel", "<f8", 3), ("w", "<f8")])


def build_port():
    subprocess.run(["make", "-s", "port"], cwd=HERE, check=True)


def build_ref():
    """Compile the reference sources (needs the reference tree; absent on GPU hosts)."""
    root = reference_root()
    if not root or not os.path.isdir(os.path.join(root, "ch4", "v3", "src")):
        return False
    subprocess.run(["make", "-s", "-j8", "ref", "REF=" + root], cwd=HERE, check=True)
    return True


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def moving_average_update(avg, samples, den):
    """Field::updateMovingAverage (Field.h:245-261) as Species::updateAverages calls it
    (Species.cpp:764-766): the sample counter restarts after 20 samples (the field is cleared),
    then avg = (den + avg (samples - 1)) / samples.  Updates avg in place; returns the counter."""
    samples += 1
    if samples > 20:
        avg[:] = 0.0
        samples = 1
    avg[:] = (den + avg * (samples - 1.0)) / samples
    return samples


def macro_particle_count(g, parts):
    """Species::computeMacroParticlesCount (Species.cpp:813-819): particles per cell, the cell
    from World::XtoIJK (World.cpp:120-133), int((x - x0) * inv_dx) per axis.  Counts in the
    linear cell order c = (k (nj-1) + j) (ni-1) + i of World::XtoC (World.cpp:134-137)."""
    x0 = np.array(g.x0[:])
    inv = np.array(g.inv_dx[:])
    ijk = ((parts["pos"] - x0) * inv).astype(np.int64)
    ci, cj, ck = g.ni - 1, g.nj - 1, g.nk - 1
    c = (ijk[:, 2] * cj + ijk[:, 1]) * ci + ijk[:, 0]
    return np.bincount(c, minlength=ci * cj * ck)


class Grid(C.Structure):
    _fields_ = [
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int),
        ("x0", C.c_double * 3), ("xm", C.c_double * 3), ("dx", C.c_double * 3), ("inv_dx", C.c_double * 3),
        ("periodic", C.c_int * 3),
        ("n_boxes", C.c_int),
        ("box_c", (C.c_double * 3) * 8), ("box_half", (C.c_double * 3) * 8),
    ]


class CollParams(C.Structure):
    _fields_ = [
        ("mass_neutral", C.c_double), ("mass_electron", C.c_double), ("E_ion_eV", C.c_double), ("B_inc", C.c_double),
        ("sigma_ion_kind", C.c_int),
        ("sig_a", C.c_double), ("sig_b", C.c_double), ("sig_c", C.c_double), ("sig_A", C.c_double),
        ("table_E", C.c_void_p), ("table_s", C.c_void_p), ("table_n", C.c_int),
        ("n_neutral", C.c_double), ("T_neutral", C.c_double), ("sigv_max", C.c_double),
    ]


class DsmcParams(C.Structure):
    _fields_ = [("mass1", C.c_double), ("mass2", C.c_double), ("mpw0", C.c_double), ("dv", C.c_double),
                ("c", C.c_double * 4)]


class ObjSpecies(C.Structure):
    _fields_ = [("neu", C.c_void_p), ("neu_ids", C.c_void_p), ("n_neu", C.c_void_p), ("cap_neu", C.c_long),
                ("neu_mpw0", C.c_double), ("spu", C.c_void_p), ("spu_ids", C.c_void_p), ("n_spu", C.c_void_p),
                ("cap_spu", C.c_long), ("spu_mpw0", C.c_double), ("sputtering", C.c_int), ("neu_qm", C.c_double),
                ("spu_qm", C.c_double), ("ef", C.c_void_p),
                ("dt_global", C.c_double)]


class MT(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("idx", C.c_int)]


class Port:
    """FP64 restatement; all arrays are numpy, node arrays flat with i fastest."""

    def __init__(self, path=PORT_SO):
        if not os.path.exists(path):
            build_port()
        L = self.lib = C.CDLL(path)
        vp, i, d, l = C.c_void_p, C.c_int, C.c_double, C.c_long
        u32 = C.c_uint32
        sig = {
            "or_grid_init": (None, [vp, i, i, i, vp, vp, vp]),
            "or_grid_add_box": (i, [vp, vp, vp]),
            "or_node_kinds": (None, [vp, i, vp]),
            "or_mt_seed": (None, [vp, u32]),
            "or_mt_u01": (d, [vp]),
            "or_philox4x32_10": (None, [vp, vp, vp]),
            "or_node_volumes": (None, [vp, vp]),
            "or_number_density_ref": (None, [vp, vp, l, vp]),
            "or_compute_ef_ref": (None, [vp, vp, vp]),
            "or_push_electrons_ref": (l, [vp, vp, l, vp, vp, d, d, d]),
            "or_push_electrons_mt": (l, [vp, vp, l, vp, vp, d, d, d, i]),
            "or_solve_gs_ref": (i, [vp, vp, vp, vp, i, d, vp, vp]),
            "or_solve_pcg_ref": (i, [vp, vp, vp, vp, i, d, i, vp, vp]),
            "or_fill_aux": (None, [vp, vp, vp]),
            "or_residual": (None, [vp, vp, vp, vp, vp, vp]),
            "or_solve_rbsor": (i, [vp, vp, vp, vp, d, d, i, vp, vp]),
            "or_solve_fpcg": (i, [vp, vp, vp, vp, d, i, vp, vp]),
            "or_sigma_coll": (d, [vp, d]),
            "or_sigma_ion": (d, [vp, d]),
            "or_sigv_majorant": (d, [vp]),
            "or_mcc_background": (l, [vp, vp, vp, vp, vp, l, vp, vp, vp, l, d, u32, u32, u32, vp]),
            "or_child_id": (C.c_uint64, [C.c_uint64, u32, u32]),
            "or_cand_draw": (u32, [C.c_uint64, u32, u32, u32]),
            "or_cand_threshold": (u32, [d]),
            "or_ntc_ionize_ref": (l, [vp, vp, vp, vp, vp, l, vp, vp, l, vp, vp, l, d, vp]),
            "or_merge_ref": (l, [vp, vp, vp, l, l, vp, d, d, d, i]),
            "or_merge_gpuform": (l, [vp, vp, vp, vp, l, l, vp, d, d, d, i, u32, u32, u32]),
            "or_load_box_thermal_ref": (l, [vp, vp, vp, l, vp, vp, d, d, d, d, d, vp, d]),
            "or_sums": (None, [vp, l, d, vp, vp, vp]),
            "or_sample_moments_ref": (None, [vp, vp, l, vp]),
            "or_gas_properties_ref": (None, [vp, vp, d, vp, vp]),
            "or_dsmc_params_init": (None, [vp, vp, d, d, d]),
            "or_dsmc_sigma": (d, [vp, d]),
            "or_dsmc_ref": (l, [vp, vp, vp, vp, l, vp, l, d, vp, vp]),
            "or_dsmc_gpuform": (l, [vp, vp, vp, vp, vp, l, d, d, u32, u32, u32, u32, vp, vp]),
            "or_push_nonelectron_ref": (l, [vp, vp, vp, l, vp, d, d, d, vp, vp]),
            "or_push_nonelectron_gpuform": (l, [vp, vp, vp, l, vp, d, d, d, vp, u32, u32, u32, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args

    # -- grid ------------------------------------------------------------------------
    def grid(self, nn, x0, xm, periodic=(0, 0, 0), boxes=()):
        g = Grid()
        self.lib.or_grid_init(C.byref(g), int(nn[0]), int(nn[1]), int(nn[2]),
                              _p(np.asarray(x0, np.float64)), _p(np.asarray(xm, np.float64)),
                              _p(np.asarray(periodic, np.int32)))
        for c, s in boxes:
            self.lib.or_grid_add_box(C.byref(g), _p(np.asarray(c, np.float64)), _p(np.asarray(s, np.float64)))
        return g

    @staticmethod
    def nv(g):
        return g.ni * g.nj * g.nk

    def node_kinds(self, g, wall_mode):
        k = np.zeros(self.nv(g), np.uint8)
        self.lib.or_node_kinds(C.byref(g), int(wall_mode), _p(k))
        return k

    def node_volumes(self, g):
        v = np.zeros(self.nv(g))
        self.lib.or_node_volumes(C.byref(g), _p(v))
        return v

    # -- rng ---------------------------------------------------------------------------
    def mt(self, seed):
        r = MT()
        self.lib.or_mt_seed(C.byref(r), int(seed))
        return r

    def philox(self, ctr, key):
        c = np.asarray(ctr, np.uint32)
        k = np.asarray(key, np.uint32)
        o = np.zeros(4, np.uint32)
        self.lib.or_philox4x32_10(_p(c), _p(k), _p(o))
        return o

    # -- particles & fields ----------------------------------------------------------------
    def number_density(self, g, parts, n=None):
        den = np.zeros(self.nv(g))
        self.lib.or_number_density_ref(C.byref(g), _p(parts), len(parts) if n is None else n, _p(den))
        return den

    def compute_ef(self, g, phi):
        ef = np.zeros((self.nv(g), 3))
        self.lib.or_compute_ef_ref(C.byref(g), _p(np.ascontiguousarray(phi, np.float64)), _p(ef))
        return ef

    def push(self, g, parts, ef, dt, charge, mass, ids=None, threads=1):
        """Pushes in place; returns the surviving count (survivors are parts[:n])."""
        ef = np.ascontiguousarray(ef, np.float64)
        if threads > 1:
            return self.lib.or_push_electrons_mt(C.byref(g), _p(parts), len(parts), _p(ids), _p(ef), dt, charge, mass,
                                                 threads)
        return self.lib.or_push_electrons_ref(C.byref(g), _p(parts), len(parts), _p(ids), _p(ef), dt, charge, mass)

    def solve_gs(self, g, kind, phi, rho, max_it, tol):
        it, l2 = C.c_int(), C.c_double()
        ok = self.lib.or_solve_gs_ref(C.byref(g), _p(kind), _p(phi), _p(rho), int(max_it), tol, C.byref(it), C.byref(l2))
        return ok, it.value, l2.value

    def solve_pcg_ref(self, g, kind, phi, rho, max_it, tol, axis_swap=1):
        it, l2 = C.c_int(), C.c_double()
        ok = self.lib.or_solve_pcg_ref(C.byref(g), _p(kind), _p(phi), _p(rho), int(max_it), tol, int(axis_swap),
                                       C.byref(it), C.byref(l2))
        return ok, it.value, l2.value

    def residual(self, g, kind, phi, rho):
        r2, b2 = C.c_double(), C.c_double()
        self.lib.or_residual(C.byref(g), _p(kind), _p(phi), _p(rho), C.byref(r2), C.byref(b2))
        return r2.value, b2.value

    def rel_residual(self, g, kind, phi, rho):
        r2, b2 = self.residual(g, kind, phi, rho)
        return float(np.sqrt(r2 / b2)) if b2 > 0 else float(np.sqrt(r2))

    def fill_aux(self, g, kind, phi):
        self.lib.or_fill_aux(C.byref(g), _p(kind), _p(phi))

    def solve_rbsor(self, g, kind, phi, rho, omega, tol_rel, max_sweeps):
        s, rel = C.c_int(), C.c_double()
        ok = self.lib.or_solve_rbsor(C.byref(g), _p(kind), _p(phi), _p(rho), omega, tol_rel, int(max_sweeps),
                                     C.byref(s), C.byref(rel))
        return ok, s.value, rel.value

    def solve_fpcg(self, g, kind, phi, rho, tol_rel, max_it):
        it, rel = C.c_int(), C.c_double()
        ok = self.lib.or_solve_fpcg(C.byref(g), _p(kind), _p(phi), _p(rho), tol_rel, int(max_it), C.byref(it),
                                    C.byref(rel))
        return ok, it.value, rel.value

    # -- collisions ----------------------------------------------------------------------
    def coll_params(self, table_E, table_s, mass_neutral, E_ion_eV, sigma_ion_kind=0, sig=(1.015e-18, 9.793, 61.81),
                    sig_A=0.0, B_inc=10.0, n_neutral=0.0, T_neutral=300.0, mass_electron=ME):
        cp = CollParams()
        cp._tE = np.ascontiguousarray(table_E, np.float64)
        cp._ts = np.ascontiguousarray(table_s, np.float64)
        cp.mass_neutral, cp.mass_electron, cp.E_ion_eV, cp.B_inc = mass_neutral, mass_electron, E_ion_eV, B_inc
        cp.sigma_ion_kind = sigma_ion_kind
        cp.sig_a, cp.sig_b, cp.sig_c = sig
        cp.sig_A = sig_A
        cp.table_E, cp.table_s, cp.table_n = cp._tE.ctypes.data, cp._ts.ctypes.data, len(cp._tE)
        cp.n_neutral, cp.T_neutral = n_neutral, T_neutral
        cp.sigv_max = self.lib.or_sigv_majorant(C.byref(cp))
        return cp

    def mcc_background(self, g, cp, ele, ele_id, n_ele, ion, ion_id, n_ion, dt, seed, step):
        ne, ni_, nion = C.c_long(n_ele), C.c_long(n_ion), C.c_long()
        ncoll = self.lib.or_mcc_background(C.byref(g), C.byref(cp), _p(ele), _p(ele_id), C.byref(ne), len(ele),
                                           _p(ion), _p(ion_id), C.byref(ni_), len(ion), dt, seed & 0xffffffff,
                                           (seed >> 32) & 0xffffffff, step, C.byref(nion))
        return ncoll, nion.value, ne.value, ni_.value

    def child_id(self, parent, step, kind):
        return int(self.lib.or_child_id(parent, step, kind))

    def ntc_ionize_ref(self, g, cp, r, neu, n_neu, ion, n_ion, ele, n_ele, dt, wsv_max):
        nn, ni_, ne = C.c_long(n_neu), C.c_long(n_ion), C.c_long(n_ele)
        w = C.c_double(wsv_max)
        nc = self.lib.or_ntc_ionize_ref(C.byref(g), C.byref(cp), C.byref(r), _p(neu), C.byref(nn), len(neu), _p(ion),
                                        C.byref(ni_), len(ion), _p(ele), C.byref(ne), len(ele), dt, C.byref(w))
        return nc, nn.value, ni_.value, ne.value, w.value

    def dsmc_params(self, g, mass1, mass2, mpw0):
        q = DsmcParams()
        self.lib.or_dsmc_params_init(C.byref(q), C.byref(g), mass1, mass2, mpw0)
        return q

    def dsmc_ref(self, g, q, r, p1, p2, dt, svmax):
        """DSMC_MEX::apply on particle arrays (p2 None: one species); returns (collisions, pairs, svmax)."""
        sv, pairs = C.c_double(svmax), C.c_long(0)
        nc = self.lib.or_dsmc_ref(C.byref(g), C.byref(q), C.byref(r), _p(p1), len(p1), _p(p2),
                                  0 if p2 is None else len(p2), dt, C.byref(sv), C.byref(pairs))
        return nc, pairs.value, sv.value

    def dsmc_gpuform(self, q, vel1, cnt1, vel2, cnt2, dt, svmax, seed, call, tag):
        """The GPU form on velocities in cell order (updated in place); returns (collisions, pairs, svmax_step)."""
        pairs, mx = C.c_long(0), C.c_double(0)
        c1 = np.ascontiguousarray(cnt1, np.int32)
        c2 = None if cnt2 is None else np.ascontiguousarray(cnt2, np.int32)
        nc = self.lib.or_dsmc_gpuform(C.byref(q), _p(vel1), _p(c1), _p(vel2), _p(c2), len(c1), dt, svmax,
                                      seed & 0xffffffff, (seed >> 32) & 0xffffffff, call, tag, C.byref(pairs),
                                      C.byref(mx))
        return nc, pairs.value, mx.value

    def _obj_species(self, neu, neu_mpw0, spu, spu_mpw0, sputtering, ef, dt_global, n_neu, n_spu,
                     neu_ids=None, spu_ids=None):
        t = ObjSpecies()
        t.neu, t.neu_ids, t.n_neu, t.cap_neu, t.neu_mpw0 = _p(neu), _p(neu_ids), C.addressof(n_neu), len(neu), neu_mpw0
        t.spu, t.spu_ids, t.n_spu = _p(spu), _p(spu_ids), C.addressof(n_spu)
        t.cap_spu, t.spu_mpw0, t.sputtering = len(spu), spu_mpw0, int(sputtering)
        t.ef, t.dt_global = _p(ef), dt_global
        return t

    def push_nonelectron_ref(self, g, r, parts, n, ef, dt, charge, mass, neu, n_neu, neu_mpw0, spu=None, n_spu=0,
                             spu_mpw0=1.0, sputtering=False, dt_global=None):
        """Species::advanceNonElectron on parts[:n]; neutrals (and sputtered particles) appended
        to neu[n_neu:] (spu[n_spu:]).  Returns (n, n_neu, n_spu)."""
        ef = np.ascontiguousarray(ef, np.float64)
        spu = neu if spu is None else spu
        a, b = C.c_long(n_neu), C.c_long(n_spu if spu is not neu else 0)
        if spu is neu:
            b = a
        t = self._obj_species(neu, neu_mpw0, spu, spu_mpw0, sputtering, ef, dt if dt_global is None else dt_global, a, b)
        created = (C.c_long * 2)()
        m = self.lib.or_push_nonelectron_ref(C.byref(g), C.byref(r), _p(parts), n, _p(ef), dt, charge, mass,
                                             C.byref(t), created)
        return m, a.value, b.value

    def push_nonelectron_gpuform(self, g, parts, ids, n, ef, dt, charge, mass, neu, neu_ids, n_neu, neu_mpw0, spu,
                                 spu_ids, n_spu, spu_mpw0, sputtering, seed, step):
        """GPU form; returns (n, n_neu, n_spu, stats)."""
        ef = np.ascontiguousarray(ef, np.float64)
        a, b = C.c_long(n_neu), C.c_long(n_spu)
        t = self._obj_species(neu, neu_mpw0, spu, spu_mpw0, sputtering, ef, dt, a, b, neu_ids, spu_ids)
        st = (C.c_long * 4)()
        m = self.lib.or_push_nonelectron_gpuform(C.byref(g), _p(parts), _p(ids), n, _p(ef), dt, charge, mass,
                                                 C.byref(t), seed & 0xffffffff, (seed >> 32) & 0xffffffff, step, st)
        return m, a.value, b.value, list(st)

    def merge_ref(self, g, r, parts, n, ef, charge, mass, dt, min_count=10):
        return self.lib.or_merge_ref(C.byref(g), C.byref(r), _p(parts), n, len(parts),
                                     _p(np.ascontiguousarray(ef, np.float64)), charge, mass, dt, min_count)

    def merge_gpuform(self, g, parts, ids, n, ef, charge, mass, dt, min_count, seed, step, cells=None):
        cl = None if cells is None else np.ascontiguousarray(cells, np.int32)
        return self.lib.or_merge_gpuform(C.byref(g), _p(parts), _p(ids), _p(cl), n, len(parts),
                                         _p(None if ef is None else np.ascontiguousarray(ef, np.float64)), charge,
                                         mass, dt, min_count, seed & 0xffffffff, (seed >> 32) & 0xffffffff, step)

    def load_box_thermal_ref(self, g, r, cap, x0, sides, num_den, T, mpw0, mass, charge, ef=None, dt=0.0):
        parts = np.zeros(cap, PARTICLE)
        n = self.lib.or_load_box_thermal_ref(C.byref(g), C.byref(r), _p(parts), cap, _p(np.asarray(x0, np.float64)),
                                             _p(np.asarray(sides, np.float64)), num_den, T, mpw0, mass, charge,
                                             _p(None if ef is None else np.ascontiguousarray(ef, np.float64)), dt)
        return parts[:n].copy()

    def sample_moments(self, g, parts, mom=None):
        mom = np.zeros(7 * self.nv(g)) if mom is None else mom
        self.lib.or_sample_moments_ref(C.byref(g), _p(parts), len(parts), _p(mom))
        return mom

    def gas_properties(self, g, mom, mass):
        vel = np.zeros((self.nv(g), 3))
        T = np.zeros(self.nv(g))
        self.lib.or_gas_properties_ref(C.byref(g), _p(mom), mass, _p(vel), _p(T))
        return vel, T

    def sums(self, parts, mass):
        c, ke = C.c_double(), C.c_double()
        mom = np.zeros(3)
        self.lib.or_sums(_p(parts), len(parts), mass, C.byref(c), _p(mom), C.byref(ke))
        return c.value, mom, ke.value


class Ref:
    """The reference's own code (oracle/_ref/libpicref.so); a World with species."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(REF_SO) and not build_ref():
                raise FileNotFoundError("reference oracle not built and reference sources absent")
            L = C.CDLL(REF_SO)
            vp, i, d, l, cp_ = C.c_void_p, C.c_int, C.c_double, C.c_long, C.c_char_p
            sig = {
                "ref_world_create": (vp, [i, i, i, vp, vp]),
                "ref_world_destroy": (None, [vp]),
                "ref_seed": (None, [C.c_uint]),
                "ref_rnd": (d, []),
                "ref_set_time": (None, [vp, d, i]),
                "ref_advance_time": (i, [vp]),
                "ref_get_ts": (i, [vp]),
                "ref_dirichlet_walls": (None, [vp, d]),
                "ref_add_rectangle": (None, [vp, vp, d, vp]),
                "ref_species_create": (i, [vp, cp_, d, d, d, d]),
                "ref_species_set": (None, [vp, i, vp, vp, vp, l]),
                "ref_species_add": (None, [vp, i, vp, vp, d]),
                "ref_species_count": (l, [vp, i]),
                "ref_species_get": (None, [vp, i, vp, vp, vp]),
                "ref_load_box_thermal": (None, [vp, i, vp, vp, d, d]),
                "ref_push_electrons": (None, [vp, i, d]),
                "ref_push_nonelectron": (None, [vp, i, i, d]),
                "ref_number_density": (None, [vp, i]),
                "ref_charge_density": (None, [vp]),
                "ref_merge": (None, [vp, i]),
                "ref_sample_moments": (None, [vp, i]),
                "ref_gas_properties": (None, [vp, i, vp, vp]),
                "ref_get_field": (None, [vp, i, vp]),
                "ref_set_field": (None, [vp, i, vp]),
                "ref_get_den": (None, [vp, i, vp]),
                "ref_update_averages": (None, [vp, i]),
                "ref_get_den_avg": (None, [vp, i, vp]),
                "ref_macro_count": (None, [vp, i, vp]),
                "ref_get_ef": (None, [vp, vp]),
                "ref_set_ef": (None, [vp, vp]),
                "ref_solver_create": (None, [vp, C.c_uint, d, i]),
                "ref_solve": (i, [vp]),
                "ref_compute_ef": (None, [vp]),
                "ref_mcmex_create": (i, [vp, i, i, i, cp_]),
                "ref_mcmex_apply": (None, [vp, d]),
                "ref_dsmc_create": (i, [vp, i, i]),
                "ref_dsmc_apply": (None, [vp, d]),
                "ref_dsmc_svmax": (d, [vp]),
                "ref_push_nonelectron_sput": (None, [vp, i, i, i, i, d]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            cls._lib = L
        return cls._lib

    def __init__(self, nn, x0, xm):
        self.L = self.lib()
        self.nn = tuple(int(v) for v in nn)
        self.h = self.L.ref_world_create(self.nn[0], self.nn[1], self.nn[2], _p(np.asarray(x0, np.float64)),
                                         _p(np.asarray(xm, np.float64)))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_world_destroy(self.h)
            self.h = None

    @property
    def nv(self):
        return self.nn[0] * self.nn[1] * self.nn[2]

    def seed(self, s):
        self.L.ref_seed(int(s))

    def species(self, name, mass, charge, mpw0, E_ion=-1.0):
        return self.L.ref_species_create(self.h, name.encode(), mass, charge, mpw0, E_ion)

    def set_particles(self, sp, parts):
        p = np.ascontiguousarray(parts)
        pos = np.ascontiguousarray(p["pos"])
        vel = np.ascontiguousarray(p["vel"])
        w = np.ascontiguousarray(p["w"])
        self.L.ref_species_set(self.h, sp, _p(pos), _p(vel), _p(w), len(p))

    def get_particles(self, sp):
        n = self.L.ref_species_count(self.h, sp)
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        w = np.zeros(n)
        self.L.ref_species_get(self.h, sp, _p(pos), _p(vel), _p(w))
        out = np.zeros(n, PARTICLE)
        out["pos"], out["vel"], out["w"] = pos, vel, w
        return out

    def field(self, which):
        out = np.zeros(self.nv)
        self.L.ref_get_field(self.h, {"phi": 0, "rho": 1, "node_vol": 2, "object_id": 3}[which], _p(out))
        return out

    def set_field(self, which, arr):
        self.L.ref_set_field(self.h, {"phi": 0, "rho": 1}[which], _p(np.ascontiguousarray(arr, np.float64)))

    def den(self, sp):
        out = np.zeros(self.nv)
        self.L.ref_get_den(self.h, sp, _p(out))
        return out

    def ef(self):
        out = np.zeros((self.nv, 3))
        self.L.ref_get_ef(self.h, _p(out))
        return out

    def set_ef(self, ef):
        self.L.ref_set_ef(self.h, _p(np.ascontiguousarray(ef, np.float64)))
