"""NCGPU on the CPU: the oracle (oracle/ncgpu_ref.py) against the fixtures
made by running the reference's own numba kernels serially
(tests/golden/ncgpu_*), and the package's TDB reader, parameters and seed
against the oracle's."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import ncgpu_ref as N
from pyphasefield_gb300.engines.ncgpu import (gibbs_table, make_seed, ncgpu_parameters,
                                              params_struct)
from pyphasefield_gb300.tdb import Database, g_eval

GOLDEN = Path(__file__).resolve().parent / "golden"
TDB = GOLDEN / "ncgpu_nicu.tdb"


@pytest.mark.parametrize("name", ["ncgpu_periodic", "ncgpu_neumann", "ncgpu_ninb"])
def test_oracle_matches_reference_kernels(name):
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    tdb = N.Tdb(GOLDEN / m["tdb"])
    p = N.tdb_params(tdb, m["dx"])
    T = np.full(z["phi0"].shape, m["T"])
    out = N.run([z["phi0"], z["q10"], z["q40"], z["c0"]], T, m["steps"], p, tdb, seed=m["seed"],
                bc=m["bc"])
    # c: the reference's dG/dc is a forward difference with step 1e-7, which
    # turns a rounding-level change of c (1e-17, from the order of the
    # operations) into 1e-11 .. 1e-10 after a few steps
    for got, key, tol in zip(out, ("phi", "q1", "q4", "c"), (1e-12, 1e-12, 1e-12, 1e-8)):
        ref = z[key]
        assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max()), key


def test_oracle_matches_reference_kernels_under_cooling():
    """A temperature falling 5 K per step (LINEAR_GRADIENT with dT/dt): the
    oracle raises T after every step as the reference's
    update_thermal_gradient kernel does, and reproduces the reference's run."""
    z = np.load(GOLDEN / "ncgpu_cooling.npz")
    m = json.loads(str(z["meta"]))
    tdb = N.Tdb(GOLDEN / m["tdb"])
    p = N.tdb_params(tdb, m["dx"])
    assert p["dt"] == m["dt"]
    out = N.run([z["phi0"], z["q10"], z["q40"], z["c0"]], z["T0"], m["steps"], p, tdb,
                seed=m["seed"], bc=m["bc"], dT_step=m["dT_step"])
    for got, key, tol in zip(out, ("phi", "q1", "q4", "c"), (1e-12, 1e-12, 1e-12, 1e-8)):
        ref = z[key]
        assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max()), key
    # the cooling matters: without it the run parts from the reference's
    still = N.run([z["phi0"], z["q10"], z["q40"], z["c0"]], z["T0"], m["steps"], p, tdb,
                  seed=m["seed"], bc=m["bc"])
    assert np.abs(still[0] - z["phi"]).max() > 1e-6


def test_tdb_reader_matches_oracle_evaluation():
    db, tdb = Database(TDB), N.Tdb(TDB)
    assert db.elements == tdb.elements == ["CU", "NI"]
    assert db.phases == tdb.phases == ["FCC_A1", "LIQUID"]
    for (ph, comp), pieces in db.params.items():
        for T in (300.0, 900.0, 1357.0, 1357.77, 1574.0, 1727.99, 1728.0, 2500.0, 3500.0):
            mine = 0.0
            for lo, hi, c in pieces:
                if lo <= T < hi:
                    mine = g_eval(c, T)
            assert mine == pytest.approx(tdb.g_pure(ph, comp, T), rel=1e-13, abs=1e-9)
    table, npieces = gibbs_table(db)
    assert table.shape == (2, 6, 4, 10)
    assert (npieces[:, :2] == 2).all() and (npieces[:, 2:] == 0).all()


def test_parameters_match_oracle():
    db, tdb = Database(TDB), N.Tdb(TDB)
    mine = ncgpu_parameters(db, 4.6e-6)
    ref = N.tdb_params(tdb, 4.6e-6)
    for k in ("d", "D_S", "D_L", "v_m", "M_qmax", "H", "y_e", "beta", "dt", "ebar"):
        assert mine[k] == pytest.approx(ref[k], rel=1e-14), k
    for k in ("L", "T_M", "S", "B", "W", "M"):
        np.testing.assert_allclose(mine[k], ref[k], rtol=1e-14)


@pytest.mark.parametrize("shape", [(40, 50), (21, 17), (12, 12)])
def test_seed_matches_oracle(shape):
    phi = np.zeros(shape)
    q1 = np.ones(shape)
    q4 = np.zeros(shape)
    make_seed(phi, q1, q4, shape[1] / 2, shape[0] / 2, np.pi / 4, 5)
    rphi, rq1, rq4, _ = N.seed_fields(shape)
    np.testing.assert_array_equal(phi, rphi)
    np.testing.assert_array_equal(q1, rq1)
    np.testing.assert_array_equal(q4, rq4)


def test_noise_is_standard_normal():
    z = N.noise_normal(3, 5, (300, 400))
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01


@pytest.mark.parametrize("name", ["ncgpu_ternary", "ncgpu_quaternary", "ncgpu_senary"])
def test_multicomponent_oracle_matches_reference_kernels(name):
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    nc = sum(1 for k in z.files if k.startswith("c0_"))
    tdb = N.Tdb(GOLDEN / m["tdb"])
    assert len(tdb.elements) == nc + 1
    p = N.tdb_params(tdb, m["dx"])
    T = np.full(z["phi0"].shape, m["T"])
    out = N.run([z["phi0"], z["q10"], z["q40"]] + [z[f"c0_{j}"] for j in range(nc)], T,
                m["steps"], p, tdb, seed=m["seed"], bc=m["bc"])
    keys = ["phi", "q1", "q4"] + [f"c_{j}" for j in range(nc)]
    for got, key, tol in zip(out, keys, [1e-10, 1e-12, 1e-12] + [1e-8] * nc):
        ref = z[key]
        assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max()), key


def test_pseudo_element_tdb_reader():
    """The six-component database: every pure-element energy and the
    derived per-component W and M agree between the package's reader and the
    oracle's."""
    path = GOLDEN / "ncgpu_6comp.tdb"
    db, tdb = Database(path), N.Tdb(path)
    assert db.elements == ["AL", "CU", "NI", "XA", "XB", "XC"]
    for (ph, comp), pieces in db.params.items():
        for T in (500.0, 1357.0, 1574.0):
            mine = [g_eval(c, T) for lo, hi, c in pieces if lo <= T < hi]
            assert mine[0] == pytest.approx(tdb.g_pure(ph, comp, T), rel=1e-13, abs=1e-9)
    mine = ncgpu_parameters(db, 4.6e-6)
    ref = N.tdb_params(tdb, 4.6e-6)
    np.testing.assert_allclose(mine["W"], ref["W"], rtol=1e-14)
    np.testing.assert_allclose(mine["M"], ref["M"], rtol=1e-14)


def test_ternary_tdb_reader():
    path = GOLDEN / "ncgpu_nicual.tdb"
    db, tdb = Database(path), N.Tdb(path)
    assert db.elements == ["AL", "CU", "NI"]
    assert db.scalar("M_Q") == pytest.approx(80000000 / 1574.0)
    for (ph, comp), pieces in db.params.items():
        for T in (500.0, 700.0, 800.0, 933.47, 1574.0):
            mine = 0.0
            for lo, hi, c in pieces:
                if lo <= T < hi:
                    mine = g_eval(c, T)
            assert mine == pytest.approx(tdb.g_pure(ph, comp, T), rel=1e-13, abs=1e-9)
    mine = ncgpu_parameters(db, 4.6e-6)
    ref = N.tdb_params(tdb, 4.6e-6)
    np.testing.assert_allclose(mine["W"], ref["W"], rtol=1e-14)
    assert mine["ebar"] == pytest.approx(ref["ebar"], rel=1e-14)


def test_more_components_than_the_tables_hold_are_rejected(tmp_path):
    text = (GOLDEN / "ncgpu_6comp.tdb").read_text()
    extra = [ln.replace("XC", "XD") for ln in text.splitlines() if "XC" in ln]
    path = tmp_path / "seven.tdb"
    path.write_text(text + "\n".join(extra) + "\n")
    db = Database(path)
    assert len(db.elements) == 7
    with pytest.raises(NotImplementedError, match="2 to 6 components"):
        ncgpu_parameters(db, 4.6e-6)


def test_params_struct_fills_every_component():
    db = Database(GOLDEN / "ncgpu_6comp.tdb")
    ud = ncgpu_parameters(db, 4.6e-6)
    p = params_struct(db, ud, 4.6e-6)
    table, npieces = gibbs_table(db)
    assert p.ncomp == 6
    for j in range(6):
        assert p.W[j] == ud["W"][j] and p.M[j] == ud["M"][j]
        for ph in range(2):
            assert p.npieces[ph][j] == npieces[ph, j] > 0
            for k in range(4):
                assert list(p.gibbs[ph][j][k]) == list(table[ph, j, k])


def _write(tmp_path, text):
    path = tmp_path / "db.tdb"
    path.write_text(text)
    return path


def test_tdb_reader_abbreviations_exponents_and_nested_functions(tmp_path):
    """Abbreviated keywords, `$` comments, a phase type suffix (LIQUID:L),
    exponents written 1.5E-003 and T**(-1), a FUNCTION whose name ends in E
    followed by a sign (GBASE+...),
    and a FUNCTION that refers to another across a range boundary (the
    pieces split where either expression changes)."""
    path = _write(tmp_path, """
$ comment line
ELEM AA FCC_A1 0 0 0 !
ELEM BB FCC_A1 0 0 0 !
FUNCT GBASE 300 +100.0-2.5E+000*T+1.5E-003*T**2; 1000 Y
   -50.0+3*T*LN(T); 3000 N !
FUNCT GSHIFT 300 GBASE+1000*T**(-1)+2*T**(-1); 3000 N !
PHASE FCC_A1 % 1 1 !
PHASE LIQUID:L % 1 1 !
PARA G(FCC_A1,AA;0) 300 GSHIFT; 3000 N !
PARA G(FCC_A1,BB;0) 300 -GBASE; 3000 N !
PARA G(LIQUID,AA;0) 300 +GBASE-10*T; 3000 N !
PARA G(LIQUID,BB;0) 300 1.0E+029*T**(-9); 3000 N !
""")
    db = Database(path)
    assert db.elements == ["AA", "BB"] and db.phases == ["FCC_A1", "LIQUID"]

    def g(ph, comp, T):
        return [g_eval(c, T) for lo, hi, c in db.params[(ph, comp)] if lo <= T < hi][0]

    import math
    for T in (400.0, 999.0, 1000.0, 2500.0):
        base = 100.0 - 2.5 * T + 1.5e-3 * T * T if T < 1000 else -50.0 + 3 * T * math.log(T)
        assert g("FCC_A1", "AA", T) == pytest.approx(base + 1000 / T + 2 / T, rel=1e-13)
        assert g("FCC_A1", "BB", T) == pytest.approx(-base, rel=1e-13)
        assert g("LIQUID", "AA", T) == pytest.approx(base - 10 * T, rel=1e-13)
        assert g("LIQUID", "BB", T) == pytest.approx(1e29 * T ** -9, rel=1e-13)
    assert [(lo, hi) for lo, hi, _ in db.params[("FCC_A1", "AA")]] == [(300.0, 1000.0),
                                                                       (1000.0, 3000.0)]


@pytest.mark.parametrize("record", [
    "PARAMETER L(LIQUID,AA,DD;0) 300 -1000; 3000 N !",   # interaction with no element DD
    "PARAMETER G(FCC_A1,AA:VA;0) 300 100; 3000 N !",     # two sublattices
    "PARAMETER G(FCC_A1,AA;1) 300 100; 3000 N !",        # order 1
    "PARAMETER G(FCC_A1,AA;0) 300 100*SIN(T); 3000 N !",  # a term outside the basis
])
def test_tdb_reader_rejects_what_the_kernel_cannot_evaluate(tmp_path, record):
    from pyphasefield_gb300.tdb import TdbError
    path = _write(tmp_path, "ELEM AA FCC_A1 0 0 0 !\nELEM BB FCC_A1 0 0 0 !\n"
                            "PHASE FCC_A1 % 1 1 !\nPHASE LIQUID % 1 1 !\n" + record + "\n")
    with pytest.raises(TdbError):
        Database(path)


def test_redlich_kister_terms_reader_oracle_and_struct():
    """The non-ideal Ni-Nb database (binary L parameters of orders 0-2 in
    both phases): the package's reader, the oracle and the C struct agree,
    and the molar Gibbs energy carries x_A x_B L_k (x_A - x_B)^k with A, B
    in the order the records write them."""
    import math
    path = GOLDEN / "ncgpu_ninb.tdb"
    db, tdb = Database(path), N.Tdb(path)
    assert db.elements == ["NB", "NI"] and len(db.excess) == 5
    T, x = 1600.0, [0.2, 0.8]
    for ph in db.phases:
        pure = sum(xi * tdb.g_pure(ph, c, T) for c, xi in zip(db.elements, x))
        ideal = pure + 8.3145 * T * sum(xi * math.log(xi) for xi in x)
        ex = 0.0
        for eph, a, b, k, pieces in db.excess:
            if eph == ph:
                xa, xb = x[db.elements.index(a)], x[db.elements.index(b)]
                L = [g_eval(c, T) for lo, hi, c in pieces if lo <= T < hi][0]
                ex += xa * xb * L * (xa - xb) ** k
        assert ex != 0.0
        assert tdb.gibbs(ph, x, T) == pytest.approx(ideal + ex, rel=1e-13)
    p = params_struct(db, ncgpu_parameters(db, 4.6e-6), 4.6e-6)
    assert p.nexcess == 5
    got = sorted((p.excess[j].phase, p.excess[j].a, p.excess[j].b, p.excess[j].order)
                 for j in range(5))
    # NI is component 1, NB component 0; FCC_A1 (the solid) is phase 0
    assert got == [(0, 1, 0, 0), (0, 1, 0, 1), (1, 1, 0, 0), (1, 1, 0, 1), (1, 1, 0, 2)]
    j = [p.excess[j].phase == 0 and p.excess[j].order == 1 for j in range(5)].index(True)
    assert p.excess[j].npieces == 1 and p.excess[j].piece[0][2] == 94812.0


def test_ternary_interactions_are_rejected(tmp_path):
    from pyphasefield_gb300.tdb import TdbError
    path = tmp_path / "t.tdb"
    path.write_text("ELEM AA FCC_A1 0 0 0 !\nELEM BB FCC_A1 0 0 0 !\nELEM CC FCC_A1 0 0 0 !\n"
                    "PHASE LIQUID % 1 1 !\n"
                    "PARAMETER L(LIQUID,AA,BB,CC;0) 300 100; 3000 N !\n")
    with pytest.raises(TdbError):
        Database(path)


@pytest.mark.parametrize("tdb_name,c0", [("ncgpu_ninb.tdb", [0.1]),
                                         ("ncgpu_6comp.tdb", [0.05, 0.2, 0.3, 0.1, 0.15])])
def test_engine_initialisation_without_gpu(tdb_name, c0):
    """NCGPUGB300 reads the database, derives the reference's parameters and
    lays out its fields before any device work."""
    from pyphasefield_gb300 import NCGPUGB300
    path = GOLDEN / tdb_name
    sim = NCGPUGB300(dimensions=[16, 20], dx=4.6e-6, tdb_path=str(path),
                     temperature_type="ISOTHERMAL", initial_T=1600.0,
                     boundary_conditions="PERIODIC",
                     user_data={"sim_type": "seed", "initial_concentration_array": c0})
    sim.initialize_fields_and_imported_data()
    tdb = N.Tdb(path)
    ref = N.tdb_params(tdb, 4.6e-6)
    assert [f.name for f in sim.fields] == ["phi", "q1", "q4"] + [
        "c_" + e for e in tdb.elements[:-1]]
    assert sim.dt == pytest.approx(ref["dt"], rel=1e-14)
    np.testing.assert_allclose(sim.user_data["W"], ref["W"], rtol=1e-14)
    np.testing.assert_allclose(sim.user_data["M"], ref["M"], rtol=1e-14)
    phi0, q10, q40, *cs = N.seed_fields((16, 20), c0=c0, ncomp=len(tdb.elements))
    np.testing.assert_array_equal(sim.fields[0].get_cells(), phi0)
    np.testing.assert_allclose(sim.fields[1].get_cells(), q10, rtol=1e-15)
    for f, c in zip(sim.fields[3:], cs):
        np.testing.assert_array_equal(f.get_cells(), c)


@pytest.mark.parametrize("name", ["ncgpu_new_periodic", "ncgpu_new_ternary"])
def test_ncgpu_new_oracle_matches_reference_kernels(name):
    """The NCGPU_new variant (per-component dG/dc and noise, phase and
    orientation noise, eqbar = 0.1 ebar, phi in [1e-4, 0.9999]) against
    Engines/NCGPU_new.py's own kernels run serially."""
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    nc = sum(1 for k in z.files if k.startswith("c0_"))
    tdb = N.Tdb(GOLDEN / m["tdb"])
    p = N.tdb_params(tdb, m["dx"], variant="NCGPU_new")
    assert p["eqbar"] == pytest.approx(0.1 * p["ebar"], rel=1e-15)
    T = np.full(z["phi0"].shape, m["T"])
    out = N.run([z["phi0"], z["q10"], z["q40"]] + [z[f"c0_{j}"] for j in range(nc)], T,
                m["steps"], p, tdb, seed=m["seed"], bc=m["bc"], variant="NCGPU_new")
    keys = ["phi", "q1", "q4"] + [f"c_{j}" for j in range(nc)]
    for got, key, tol in zip(out, keys, [1e-10, 1e-12, 1e-12] + [1e-8] * nc):
        ref = z[key]
        assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max()), key


def test_noise_streams_are_distinct_and_stream_zero_is_the_ncgpu_stream():
    a = N.noise_normal(5, 2, (9, 11))
    np.testing.assert_array_equal(a, N.noise_normal(5, 2, (9, 11), stream=0))
    d = N.noise_new(5, 2, (9, 11), 2)
    np.testing.assert_array_equal(d["c"][0], a)
    fields = d["c"] + [d["phi"], d["q1"], d["q4"]]
    for i in range(len(fields)):
        for j in range(i + 1, len(fields)):
            assert np.abs(fields[i] - fields[j]).max() > 0.1


def test_ncgpu_new_engine_initialisation_without_gpu():
    """NCGPU_newGB300: eqbar = 0.1 ebar, noise amplitudes default to 1, the
    orientation starts at melt_angle, "seeds" places the requested number
    of seeds from the engine's seeded generator (reproducible), and a wrong
    initial_concentration_array falls back to 1 / N as in the reference."""
    from pyphasefield_gb300 import NCGPU_newGB300
    path = GOLDEN / "ncgpu_nicual.tdb"

    def make(**ud):
        sim = NCGPU_newGB300(dimensions=[40, 44], dx=4.6e-6, tdb_path=str(path),
                             temperature_type="ISOTHERMAL", initial_T=1574.0,
                             user_data=dict(ud, seed=3))
        sim.initialize_fields_and_imported_data()
        return sim

    a = make(sim_type="seeds", number_of_seeds=3, melt_angle=0.3,
             initial_concentration_array=[0.1])
    assert a.user_data["eqbar"] == pytest.approx(0.1 * a.user_data["ebar"], rel=1e-15)
    assert (a.user_data["noise_phi"], a.user_data["noise_c"], a.user_data["noise_q"]) == \
        (1.0, 1.0, 1.0)
    phi, q1 = a.fields[0].get_cells(), a.fields[1].get_cells()
    assert phi.sum() > 0 and np.isclose(q1[phi == 0], np.cos(0.15)).mean() > 0.5
    for f in a.fields[3:]:
        np.testing.assert_array_equal(f.get_cells(), 1.0 / 3)  # wrong length: 1 / N
    b = make(sim_type="seeds", number_of_seeds=3, melt_angle=0.3)
    np.testing.assert_array_equal(b.fields[0].get_cells(), phi)
    melt = make(melt_angle=0.3)
    assert melt.fields[0].get_cells().sum() == 0
    np.testing.assert_allclose(melt.fields[1].get_cells(), np.cos(0.15), rtol=1e-15)


@pytest.mark.parametrize("name,variant", [("ncgpu_periodic", "NCGPU"),
                                          ("ncgpu_new_periodic", "NCGPU_new"),
                                          ("ncgpu_new_ternary", "NCGPU_new")])
def test_float32_emulation_sets_the_float_tolerances(name, variant):
    """The kernel's float32 arithmetic repeated on the CPU (oracle/ncgpu_f32)
    against the reference's kernels: within the GPU tests' float tolerance
    (1e-5), except q4 of the binary NCGPU_new case, where one interface
    cell's |grad q| falls on the other side of the beta clamp at step 2
    (~1.3e-4, the GPU measured the same): the GPU test holds that case to
    1e-3."""
    from oracle import ncgpu_f32 as E
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    tdb = N.Tdb(GOLDEN / m["tdb"])
    p = N.tdb_params(tdb, m["dx"], variant=variant)
    cks = sorted(k for k in z.files if k.startswith("c0_"))
    c0 = [z["c0"]] if "c0" in z.files else [z[k] for k in cks]
    keys = ["phi", "q1", "q4"] + (["c"] if "c" in z.files else [k.replace("c0_", "c_") for k in cks])
    with np.errstate(all="ignore"):
        out = E.run([z["phi0"], z["q10"], z["q40"]] + c0, np.full(z["phi0"].shape, m["T"]),
                    m["steps"], p, tdb, m["seed"], m["bc"], variant)
    for got, key in zip(out, keys):
        err = np.linalg.norm(got - z[key]) / np.linalg.norm(z[key])
        if (name, key) == ("ncgpu_new_periodic", "q4"):
            assert 5e-5 < err < 1e-3, err
        else:
            assert err < 1e-5, (key, err)


@pytest.mark.parametrize("tdb_name", ["ncgpu_nicu.tdb", "ncgpu_nicual.tdb", "ncgpu_4comp.tdb",
                                      "ncgpu_6comp.tdb", "ncgpu_ninb.tdb"])
def test_fixture_databases_survive_re_emission(tmp_path, tdb_name):
    """The fixture script re-emits parsed databases (every temperature range
    of every G and L parameter): written again, a database evaluates the
    same."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    src = GOLDEN / tdb_name
    out = tmp_path / tdb_name
    mg.write_tdb(N.Tdb(src), out)
    a, b = Database(src), Database(out)
    assert a.elements == b.elements and a.phases == b.phases
    assert sorted(a.params) == sorted(b.params)
    assert [e[:4] for e in a.excess] == [e[:4] for e in b.excess]
    for T in (400.0, 1200.0, 1574.0, 1800.0, 2800.0):
        for key in a.params:
            va = [g_eval(c, T) for lo, hi, c in a.params[key] if lo <= T < hi]
            vb = [g_eval(c, T) for lo, hi, c in b.params[key] if lo <= T < hi]
            assert va == pytest.approx(vb, rel=1e-14), (key, T)
        for ea, eb in zip(a.excess, b.excess):
            va = [g_eval(c, T) for lo, hi, c in ea[4] if lo <= T < hi]
            vb = [g_eval(c, T) for lo, hi, c in eb[4] if lo <= T < hi]
            assert va == pytest.approx(vb, rel=1e-14)


@pytest.mark.parametrize("dims", [[10, 10], [5, 5], [20, 1]])
def test_reference_ncomponent_shapes_initialise(dims):
    """The reference's NComponent tests (tests/test_NComponent.py: 10 x 10,
    a 5 x 5 grid smaller than the seed, a 20 x 1 strip) on the Ni-Cu
    database: the seed wraps around the grid as make_seed does, the fields
    and parameters are laid out without a GPU."""
    from pyphasefield_gb300 import NCGPUGB300
    sim = NCGPUGB300(dimensions=dims, dx=4.6e-6, tdb_path=str(TDB),
                     temperature_type="ISOTHERMAL", initial_T=1574.0,
                     user_data={"sim_type": "seed", "initial_concentration_array": [0.40831]})
    sim.initialize_fields_and_imported_data()
    phi0, q10, q40, c0 = N.seed_fields(tuple(dims), c0=0.40831)
    np.testing.assert_array_equal(sim.fields[0].get_cells(), phi0)
    np.testing.assert_allclose(sim.fields[2].get_cells(), q40, rtol=1e-15, atol=0)
    assert [f.name for f in sim.fields] == ["phi", "q1", "q4", "c_CU"]
