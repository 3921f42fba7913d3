"""Regenerates the golden fixtures from the reference's own ch4/v3 code.

Runs oracle/_ref/libpicref.so (the reference sources compiled unmodified by oracle/Makefile,
driven through ref_harness.cpp) on small seeded cases and stores inputs and outputs as .npz
files next to this script.  Needs the reference tree (PIC_REFERENCE_ROOT, else the default of
oracle/Makefile); the fixtures themselves travel with the repository.

    python tests/golden/make_golden.py [case ...]     (no case: all of them)
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

E_ION_O_J = 1313.9 * 1000 / 6.02214076e23  # main.cpp:103


def v3(*a):
    return (C.c_double * 3)(*a)


def parts_arrays(p):
    return dict(pos=p["pos"].copy(), vel=p["vel"].copy(), w=p["w"].copy())


def case_push_deposit():
    nn, x0, xm = (11, 9, 13), (-0.01, 0.0, 0.0), (0.01, 0.016, 0.03)
    R = O.Ref(nn, x0, xm)
    R.seed(7)
    e = R.species("e-", O.ME, -O.QE, 100.0)
    R.L.ref_load_box_thermal(R.h, e, v3(0, 0.008, 0.015), v3(0.018, 0.014, 0.028), 1e10, 30000.0)
    loaded = R.get_particles(e)
    rng = np.random.default_rng(11)
    ef = rng.normal(size=(R.nv, 3)) * 2e3
    R.set_ef(ef)
    R.L.ref_set_time(R.h, 1e-11, 10)
    R.L.ref_push_electrons(R.h, e, 1e-11)
    pushed = R.get_particles(e)
    R.L.ref_number_density(R.h, e)
    den = R.den(e)
    # Species::sampleMoments twice (it accumulates) + computeGasProperties
    R.L.ref_sample_moments(R.h, e)
    R.L.ref_sample_moments(R.h, e)
    gvel = np.zeros((R.nv, 3))
    gT = np.zeros(R.nv)
    R.L.ref_gas_properties(R.h, e, gvel.ctypes.data_as(C.c_void_p), gT.ctypes.data_as(C.c_void_p))
    out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), ef=ef, dt=np.array(1e-11))
    out.update({"in_" + k: v for k, v in parts_arrays(loaded).items()})
    out.update({"out_" + k: v for k, v in parts_arrays(pushed).items()})
    out["den"] = den
    out["gas_vel"], out["gas_T"] = gvel, gT
    return out


def case_poisson():
    nn, x0, xm = (11, 9, 13), (-0.01, 0.0, 0.0), (0.01, 0.016, 0.03)
    rng = np.random.default_rng(5)
    rho = rng.normal(size=int(np.prod(nn))) * 1e-8
    out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), rho=rho)
    box_c, box_s = (0.0, 0.008, 0.0), (0.02, 0.016, 0.006)
    out["box_c"], out["box_s"], out["box_phi"] = np.array(box_c), np.array(box_s), np.array(100.0)
    for mode in ("dirichlet", "v3box"):
        for st, name in ((0, "gs"), (1, "pcg")):
            R = O.Ref(nn, x0, xm)
            if mode == "dirichlet":
                R.L.ref_dirichlet_walls(R.h, 0.0)
            else:
                R.L.ref_add_rectangle(R.h, v3(*box_c), 100.0, v3(*box_s))
            R.set_field("rho", rho)
            R.L.ref_solver_create(R.h, 20000 if st == 0 else 2000, 1e-6, st)
            ok = R.L.ref_solve(R.h)
            R.L.ref_compute_ef(R.h)
            out[f"{mode}_{name}_phi"] = R.field("phi")
            out[f"{mode}_{name}_ef"] = R.ef()
            out[f"{mode}_{name}_ok"] = np.array(ok)
    return out


def sigma_table():
    E = np.geomspace(0.1, 1000.0, 60)
    S = 5e-20 / np.sqrt(1 + E / 50.0) + 1e-20
    return E, S


def write_table(E, S):
    tf = tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False)
    for a, b in zip(E, S):
        tf.write("%.17g %.17g\n" % (a, b))
    tf.close()
    return tf.name


def case_ntc():
    """MC_MEX_Ionization::apply twice on neutral macroparticles (Interactions.cpp:600-762)."""
    nn, x0, xm = (5, 5, 6), (0.0, 0.0, 0.0), (0.004, 0.004, 0.005)
    E, S = sigma_table()
    path = write_table(E, S)
    try:
        R = O.Ref(nn, x0, xm)
        R.seed(3)
        neu = R.species("O", 16 * O.AMU, 0.0, 5e11, E_ION_O_J)
        ion = R.species("O+", 16 * O.AMU, O.QE, 100.0)
        ele = R.species("e-", O.ME, -O.QE, 100.0)
        c, s = v3(0.002, 0.002, 0.0025), v3(0.004, 0.004, 0.005)
        R.L.ref_load_box_thermal(R.h, ele, c, s, 2.5e12, 11604 * 300.0)  # 2000 electrons
        R.L.ref_load_box_thermal(R.h, neu, c, s, 1.25e22, 300.0)  # 2000 neutrals
        assert R.L.ref_mcmex_create(R.h, neu, ion, ele, path.encode()) == 0
        out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), table_E=E, table_s=S, seed=np.array(3),
                   dt=np.array(1e-9), wsv0=np.array(1e-14 * 5e11))
        out.update({"ele0_" + k: v for k, v in parts_arrays(R.get_particles(ele)).items()})
        out.update({"neu0_" + k: v for k, v in parts_arrays(R.get_particles(neu)).items()})
        R.L.ref_set_time(R.h, 1e-9, 10)
        for it in range(2):
            R.L.ref_mcmex_apply(R.h, 1e-9)
            for nm, sp in (("ele", ele), ("neu", neu), ("ion", ion)):
                out.update({f"{nm}{it + 1}_" + k: v for k, v in parts_arrays(R.get_particles(sp)).items()})
        return out
    finally:
        os.unlink(path)


def case_merge():
    """Species::merge (Species.cpp:981-1145) on 600 electrons per cell."""
    nn, x0, xm = (3, 2, 2), (0.0, 0.0, 0.0), (0.002, 0.001, 0.001)
    R = O.Ref(nn, x0, xm)
    R.seed(9)
    ele = R.species("e-", O.ME, -O.QE, 100.0)
    R.L.ref_load_box_thermal(R.h, ele, v3(0.001, 0.0005, 0.0005), v3(0.002, 0.001, 0.001), 6e13, 11604 * 2.0)
    rng = np.random.default_rng(2)
    ef = rng.normal(size=(R.nv, 3)) * 1e3
    R.set_ef(ef)
    R.L.ref_set_time(R.h, 1e-12, 10)
    out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), ef=ef, dt=np.array(1e-12), seed=np.array(9))
    out.update({"in_" + k: v for k, v in parts_arrays(R.get_particles(ele)).items()})
    R.L.ref_merge(R.h, ele)
    out.update({"out_" + k: v for k, v in parts_arrays(R.get_particles(ele)).items()})
    return out


def case_dsmc():
    """DSMC_MEX::apply (Interactions.cpp:143-284): one species three times, then two species twice.

    The loads draw from the global RNG; it is reseeded (dsmc_seed) before the first apply so that a
    restatement can start from the stored particles."""
    nn, x0, xm = (5, 5, 5), (0.0, 0.0, 0.0), (0.004, 0.004, 0.004)
    mpw0, dt = 3.2e10, 1e-5
    R = O.Ref(nn, x0, xm)
    R.seed(5)
    a = R.species("O", 16 * O.AMU, 0.0, mpw0)
    b = R.species("O2", 32 * O.AMU, 0.0, mpw0)
    c, s = v3(0.002, 0.002, 0.002), v3(0.004, 0.004, 0.004)
    R.L.ref_load_box_thermal(R.h, a, c, s, 1e21, 300.0)  # 2000 particles, ~31 per cell
    R.L.ref_load_box_thermal(R.h, b, c, s, 1e21, 900.0)
    out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), mpw0=np.array(mpw0), dt=np.array(dt),
               dsmc_seed=np.array(77))
    out.update({"a0_" + k: v for k, v in parts_arrays(R.get_particles(a)).items()})
    out.update({"b0_" + k: v for k, v in parts_arrays(R.get_particles(b)).items()})
    R.seed(77)
    assert R.L.ref_dsmc_create(R.h, a, -1) == 0
    for it in range(3):
        R.L.ref_dsmc_apply(R.h, dt)
        out[f"one{it + 1}_vel"] = R.get_particles(a)["vel"].copy()
        out[f"one{it + 1}_svmax"] = np.array(R.L.ref_dsmc_svmax(R.h))
    assert R.L.ref_dsmc_create(R.h, a, b) == 0
    for it in range(2):
        R.L.ref_dsmc_apply(R.h, dt)
        out[f"two{it + 1}_vel_a"] = R.get_particles(a)["vel"].copy()
        out[f"two{it + 1}_vel_b"] = R.get_particles(b)["vel"].copy()
        out[f"two{it + 1}_svmax"] = np.array(R.L.ref_dsmc_svmax(R.h))
    return out


def case_objects():
    """Species::advanceNonElectron with a Rectangle (Species.cpp:45-256): neutrals bounce, ions are
    neutralised with sputtering on.  Three steps; each pushes the neutrals, then the ions.  The
    global RNG is reseeded (obj_seed) after the loads."""
    nn, x0, xm = (11, 11, 11), (0.0, 0.0, 0.0), (0.01, 0.01, 0.01)
    R = O.Ref(nn, x0, xm)
    R.L.ref_add_rectangle(R.h, v3(0.005, 0.005, 0.005), 0.0, v3(0.004, 0.004, 0.004))
    R.seed(13)
    neu = R.species("O", 16 * O.AMU, 0.0, 1e9)
    ion = R.species("O+", 16 * O.AMU, O.QE, 1e10)
    spu = R.species("Sp", 16 * O.AMU, 0.0, 5e8)
    c, s = v3(0.005, 0.005, 0.005), v3(0.01, 0.01, 0.01)
    R.L.ref_load_box_thermal(R.h, neu, c, s, 2e18, 300.0)  # ~1900 outside the box
    R.L.ref_load_box_thermal(R.h, ion, c, s, 1e19, 30000.0)
    rng = np.random.default_rng(4)
    ef = rng.normal(size=(R.nv, 3)) * 1e3
    R.set_ef(ef)
    dt_n, dt_i = 2e-6, 2e-7
    R.L.ref_set_time(R.h, dt_i, 10)
    out = dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), ef=ef, dt_n=np.array(dt_n), dt_i=np.array(dt_i),
               box_c=np.array([0.005] * 3), box_s=np.array([0.004] * 3), obj_seed=np.array(21))
    out.update({"neu0_" + k: v for k, v in parts_arrays(R.get_particles(neu)).items()})
    out.update({"ion0_" + k: v for k, v in parts_arrays(R.get_particles(ion)).items()})
    R.seed(21)
    for it in range(3):
        R.L.ref_push_nonelectron_sput(R.h, neu, neu, neu, 0, dt_n)
        R.L.ref_push_nonelectron_sput(R.h, ion, neu, spu, 1, dt_i)
        for nm, sp in (("neu", neu), ("ion", ion), ("spu", spu)):
            out.update({f"{nm}{it + 1}_" + k: v for k, v in parts_arrays(R.get_particles(sp)).items()})
    return out


def case_averages():
    """Species::updateAverages (the Field.h:245-261 moving average, which restarts after 20
    samples) over 45 number densities of changing particle sets, and
    Species::computeMacroParticlesCount (Species.cpp:813-819) of the last set."""
    nn, x0, xm = (6, 5, 7), (0.0, 0.0, 0.0), (0.005, 0.004, 0.006)
    R = O.Ref(nn, x0, xm)
    ele = R.species("e-", O.ME, -O.QE, 10.0)
    rng = np.random.default_rng(3)
    dens, avgs = [], []
    for it in range(45):
        n = 500 + 20 * it
        p = np.zeros(n, O.PARTICLE)
        p["pos"] = rng.uniform(0, 1, (n, 3)) * np.array(xm) * 0.999999
        p["vel"] = rng.normal(size=(n, 3)) * 1e5
        p["w"] = rng.lognormal(np.log(10.0), 0.5, n)
        R.set_particles(ele, p)
        R.L.ref_number_density(R.h, ele)
        R.L.ref_update_averages(R.h, ele)
        den = np.zeros(R.nv)
        avg = np.zeros(R.nv)
        R.L.ref_get_den(R.h, ele, den.ctypes.data_as(C.c_void_p))
        R.L.ref_get_den_avg(R.h, ele, avg.ctypes.data_as(C.c_void_p))
        dens.append(den)
        avgs.append(avg)
    cnt = np.zeros((nn[0] - 1) * (nn[1] - 1) * (nn[2] - 1))  # a cell-sized field (Species.cpp:32)
    R.L.ref_macro_count(R.h, ele, cnt.ctypes.data_as(C.c_void_p))
    return dict(nn=np.array(nn), x0=np.array(x0), xm=np.array(xm), den=np.array(dens), den_avg=np.array(avgs),
                last_pos=p["pos"].copy(), macro_count=cnt)


def main():
    cases = (("push_deposit", case_push_deposit), ("poisson", case_poisson), ("ntc", case_ntc), ("merge", case_merge),
             ("dsmc", case_dsmc), ("objects", case_objects), ("averages", case_averages))
    only = set(sys.argv[1:])
    for name, fn in cases:
        if only and name not in only:
            continue
        d = fn()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **d)
        print(name, os.path.getsize(path), "bytes", {k: np.shape(v) for k, v in d.items() if np.ndim(v) and len(v) > 50})


if __name__ == "__main__":
    main()
