"""Generates tests/golden/*.npz from pyphasefield's OWN engine functions.

Run in a checkout that has the reference (see oracle/refshim.py):
    python tests/golden/make_golden.py
Each fixture stores the initial interior field(s), the run parameters, and
the interior after `steps` steps computed by the reference's numpy engine
(engine_ExplicitDiffusion, engine_CahnAllenExplicit,
engine_CahnHilliardExplicit, engine_Warren1995, the implicit /
Crank-Nicolson / IMEX engines) driven by oracle.refshim, or by the
reference's NCGPU and NCGPU_new numba kernels run serially under a stand-in
numba module (ncgpu_* fixtures, with the databases they read re-emitted
beside them). The inputs are seeded synthetic fields (numpy default_rng).
Parts can be regenerated alone: `python tests/golden/make_golden.py
ncgpu_multicomponent | ncgpu_excess | ncgpu_new`.
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import refshim, restate  # noqa: E402
from oracle.philox import noise_uniform  # noqa: E402


def disk_seed(shape, center, r):
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi = np.ones(shape)
    phi[(yy - center[0]) ** 2 + (xx - center[1]) ** 2 < r * r] = 0.0
    return phi


def save(name, meta, **arrays):
    np.savez_compressed(HERE / f"{name}.npz", meta=json.dumps(meta), **arrays)
    print(name, {k: v.shape for k, v in arrays.items()})


def write_tdb(tdb, path):
    """The FUNCTION and PARAMETER records the NCGPU fixtures use, re-emitted
    from the parsed database (so that a machine without the reference
    checkout reads the same thermodynamic data)."""
    lines = ["$ " + "-".join(tdb.elements) + " records used by the NCGPU fixtures "
             "(written by tests/golden/make_golden.py)"]
    for el in tdb.elements:
        lines.append(f"ELEMENT {el} FCC_A1 0 0 0 !")
    for name, pieces in tdb.functions.items():
        body = f"{pieces[0][0]!r} {pieces[0][2]}"
        for k, (lo, hi, expr) in enumerate(pieces):
            more = k + 1 < len(pieces)
            body += f"; {hi!r} " + (f"Y {pieces[k + 1][2]}" if more else "N")
        lines.append(f"FUNCTION {name} {body} !")
    def ranges(pieces):
        body = f"{pieces[0][0]!r} {pieces[0][2].replace('#', '')}"
        for k, (lo, hi, expr) in enumerate(pieces):
            more = k + 1 < len(pieces)
            body += f"; {hi!r} " + (f"Y {pieces[k + 1][2].replace('#', '')}" if more else "N")
        return body

    for ph in tdb.phases:
        lines.append(f"PHASE {ph} % 1 1 !")
        for (pph, comp), pieces in tdb.params.items():
            if pph == ph:
                lines.append(f"PARAMETER G({ph},{comp};0) {ranges(pieces)} !")
        for pph, a, b, k, pieces in getattr(tdb, "excess", []):
            if pph == ph:
                lines.append(f"PARAMETER L({ph},{a},{b};{k}) {ranges(pieces)} !")
    Path(path).write_text("\n".join(lines) + "\n")


def single(name, model, c0, steps, bc, dx, dt, values=None, **params):
    if model == "cahn_hilliard":
        out = refshim.run_cahn_hilliard_extended(c0, steps, bc, dx, dt, params["M"],
                                                 params["epsilon"])
    else:
        out = refshim.run_single(model, c0, steps, bc, dx, dt, values=values, **params)
    meta = dict(model=model, steps=steps, bc=bc, dx=dx, dt=dt, values=values, params=params)
    save(name, meta, c0=c0, out=out)


def main():
    # this script reads the reference checkout; PPF_REFERENCE_ROOT names it
    os.environ.setdefault("PPF_REFERENCE_ROOT", "/root/reference/pyphasefield")
    if not refshim.available():
        raise SystemExit("reference checkout not found (set PPF_REFERENCE_ROOT)")
    rng = np.random.default_rng(20240601)
    single("diffusion_2d_periodic", "diffusion", 0.5 + 0.01 * rng.standard_normal((24, 20)),
           10, "PERIODIC", 1.0, 0.2, D=1.0)
    single("diffusion_1d_neumann", "diffusion", rng.random(40), 10, "NEUMANN", 1.0, 0.5, D=0.1)
    single("diffusion_3d_mixed", "diffusion", rng.random((10, 9, 8)), 4,
           ["NEUMANN", "DIRCHLET", "PERIODIC"], 0.5, 0.01,
           values=[[[0.1, -0.2], [0.3, 0.4], [0.0, 0.0]]], D=1.0)
    single("diffusion_2d_dirichlet", "diffusion", rng.random((13, 17)), 6,
           ["DIRCHLET", "NEUMANN"], 1.0, 0.2, values=[[[0.25, 0.75], [0.0, 0.0]]], D=1.0)
    single("allen_cahn_2d_neumann", "allen_cahn", rng.random((16, 18)), 8, "NEUMANN", 1.0, 0.1,
           M=0.1, epsilon=1.0, W=1.0)
    single("allen_cahn_3d_periodic", "allen_cahn", rng.random((8, 10, 12)), 4, "PERIODIC", 1.0,
           0.05, M=0.1, epsilon=1.0, W=1.0)
    single("cahn_hilliard_3d_periodic", "cahn_hilliard",
           0.5 + rng.uniform(-0.05, 0.05, (10, 11, 12)), 3, "PERIODIC", 1.0, 0.01, M=1.0,
           epsilon=1.0)
    single("cahn_hilliard_2d_neumann", "cahn_hilliard",
           0.5 + rng.uniform(-0.2, 0.2, (14, 16)), 3, "NEUMANN", 1.0, 0.01, M=1.0, epsilon=1.0)
    single("cahn_hilliard_3d_mixed", "cahn_hilliard",
           0.5 + rng.uniform(-0.2, 0.2, (9, 12, 10)), 2, ["PERIODIC", "NEUMANN", "PERIODIC"],
           1.0, 0.01, M=1.0, epsilon=1.0)

    # implicit / Crank-Nicolson diffusion (Engines/Diffusion.py:210-633);
    # their own generator keeps the fixtures below unchanged
    irng = np.random.default_rng(20240602)
    for name, fn, shape, steps, D, dt, dx_ in [
        ("implicit_1d", "engine_ImplicitDiffusion1D", (40,), 3, 1.0, 0.5, 1.0),
        ("crank_nicolson_1d", "engine_CrankNicolsonDiffusion1D", (37,), 3, 1.0, 2.0, 1.0),
        ("implicit_2d", "engine_ImplicitDiffusion2D", (12, 10), 2, 0.7, 1.0, 1.0),
        ("crank_nicolson_2d", "engine_CrankNicolsonDiffusion2D", (9, 14), 2, 1.0, 3.0, 1.0),
        ("implicit_3d", "engine_ImplicitDiffusion3D", (6, 7, 5), 2, 0.5, 1.0, 0.8),
        ("crank_nicolson_3d", "engine_CrankNicolsonDiffusion3D", (5, 6, 8), 2, 1.0, 0.4, 1.0),
        ("implicit_2d_adi", "engine_ImplicitDiffusion2D_ADI", (24, 20), 3, 1.0, 2.0, 1.0),
        ("crank_nicolson_2d_adi", "engine_CrankNicolsonDiffusion2D_ADI", (19, 23), 3, 1.0, 0.8, 1.0),
        ("implicit_3d_adi", "engine_ImplicitDiffusion3D_ADI", (8, 10, 12), 2, 1.0, 5.0, 1.0),
        ("crank_nicolson_3d_adi", "engine_CrankNicolsonDiffusion3D_ADI", (9, 7, 11), 2, 0.3, 1.0, 0.5),
        ("implicit_2d_adi_gmres", "engine_ImplicitDiffusion2D_ADI_GMRES", (16, 12), 2, 1.0, 1.0, 1.0),
    ]:
        c0 = irng.random(shape)
        out = refshim.run_implicit(fn, c0, steps, D, dt, dx_)
        meta = dict(model="diffusion_implicit", function=fn, steps=steps, D=D, dt=dt, dx=dx_,
                    solver="crank-nicolson" if "CrankNicolson" in fn else "implicit",
                    adi="ADI" in fn, gmres="GMRES" in fn)
        save(name, meta, c0=c0, out=out)

    # implicit / Crank-Nicolson / IMEX Allen-Cahn and Cahn-Hilliard
    # (CahnAllen.py:137-267, CahnHilliard.py:148-227)
    prng = np.random.default_rng(20240603)
    ud = dict(M=0.7, W=1.3, epsilon=1.1)
    # the full 2-D system (the GMRES engine) runs with dt = 0.1 here (16 W M
    # dt < 4: the library's Chebyshev solve) and, in phase_indefinite, with
    # dt = 0.5 (beyond it: MINRES); the others with dt = 0.3
    for name, module, fn, shape, solver, adi, gm in [
        ("phase_implicit_ac_1d", "CahnAllen", "engine_CahnAllenImplicit1D", (40,), "implicit",
         False, False),
        ("phase_implicit_ac_1d_gmres", "CahnAllen", "engine_CahnAllenImplicit1D_GMRES", (40,),
         "implicit", False, True),
        ("phase_implicit_ac_2d_gmres", "CahnAllen", "engine_CahnAllenImplicit2D_GMRES", (9, 8),
         "implicit", False, True),
        ("phase_implicit_ac_2d_adi", "CahnAllen", "engine_CahnAllenImplicit2D_ADI", (20, 24),
         "implicit", True, False),
        ("phase_implicit_ac_2d_adi_gmres", "CahnAllen", "engine_CahnAllenImplicit2D_ADI_GMRES",
         (12, 10), "implicit", True, True),
        ("phase_implicit_ac_2d_cn_adi", "CahnAllen", "engine_CahnAllenCrankNicolson2D_ADI",
         (19, 21), "crank-nicolson", True, False),
        ("phase_implicit_ac_3d_adi", "CahnAllen", "engine_CahnAllenImplicit3D_ADI", (6, 8, 10),
         "implicit", True, False),
        ("phase_implicit_ac_1d_imex", "CahnAllen", "engine_CahnAllenIMEX1D", (40,), "imex",
         False, False),
        ("phase_implicit_ch_1d", "CahnHilliard", "engine_CahnHilliardImplicit1D", (40,),
         "implicit", False, False),
        ("phase_implicit_ch_1d_cn", "CahnHilliard", "engine_CahnHilliardCrankNicolson1D", (36,),
         "crank-nicolson", False, False),
    ]:
        c0 = 0.5 + 0.4 * (prng.random(shape) - 0.5)
        dt, dx_ = (0.1 if name == "phase_implicit_ac_2d_gmres" else 0.3), 1.2
        out = refshim.run_implicit(fn, c0, 3, None, dt, dx_, module=module, user_data=ud)
        meta = dict(model="allen_cahn" if module == "CahnAllen" else "cahn_hilliard",
                    function=fn, steps=3, dt=dt, dx=dx_, solver=solver, adi=adi, gmres=gm,
                    params=ud)
        save(name, meta, c0=c0, out=out)
    phase_indefinite()

    # NCGPU (Engines/NCGPU.py): the reference's numba kernels run serially
    # under a stand-in numba module, Ni-Cu ideal TDB of the reference
    from oracle import ncgpu_ref
    tdb_path = refshim.reference_root() / "pyphasefield" / "examples" / "Ni-Cu_Ideal.tdb"
    tdb = ncgpu_ref.Tdb(tdb_path)
    write_tdb(tdb, HERE / "ncgpu_nicu.tdb")
    tdb = ncgpu_ref.Tdb(HERE / "ncgpu_nicu.tdb")
    nrng = np.random.default_rng(20240604)
    for name, shape, bc, steps, seed in [("ncgpu_periodic", (24, 20), "PERIODIC", 4, 7),
                                         ("ncgpu_neumann", (20, 22), "NEUMANN", 3, 11)]:
        p = ncgpu_ref.tdb_params(tdb, 4.6e-6)
        phi0, q10, q40, c0 = ncgpu_ref.seed_fields(shape, c0=0.40831)
        c0 = c0 + nrng.uniform(-1e-3, 1e-3, shape)
        T = np.full(shape, 1574.0)
        noise = [ncgpu_ref.noise_normal(seed, s, shape) for s in range(steps)]
        out = refshim.run_ncgpu(phi0, q10, q40, c0, T, steps, p, tdb, noise, bc)
        meta = dict(model="ncgpu", steps=steps, bc=bc, seed=seed, dx=4.6e-6, T=1574.0,
                    tdb="ncgpu_nicu.tdb")
        save(name, meta, phi0=phi0, q10=q10, q40=q40, c0=c0, phi=out[0], q1=out[1], q4=out[2],
             c=out[3])

    # NCGPU with three components (the reference's tests/Ni-Cu-Al_Ideal.tdb)
    tdb3_path = refshim.reference_root() / "pyphasefield" / "tests" / "Ni-Cu-Al_Ideal.tdb"
    write_tdb(ncgpu_ref.Tdb(tdb3_path), HERE / "ncgpu_nicual.tdb")
    tdb3 = ncgpu_ref.Tdb(HERE / "ncgpu_nicual.tdb")
    shape = (18, 16)
    p3 = ncgpu_ref.tdb_params(tdb3, 4.6e-6)
    phi0, q10, q40, ca, cb = ncgpu_ref.seed_fields(shape, c0=[0.05, 0.4], ncomp=3)
    ca = ca + nrng.uniform(-1e-3, 1e-3, shape)
    cb = cb + nrng.uniform(-1e-3, 1e-3, shape)
    T = np.full(shape, 1574.0)
    noise = [ncgpu_ref.noise_normal(5, s, shape) for s in range(3)]
    out = refshim.run_ncgpu(phi0, q10, q40, [ca, cb], T, 3, p3, tdb3, noise, "PERIODIC")
    meta = dict(model="ncgpu", steps=3, bc="PERIODIC", seed=5, dx=4.6e-6, T=1574.0,
                tdb="ncgpu_nicual.tdb")
    save("ncgpu_ternary", meta, phi0=phi0, q10=q10, q40=q40, c0_0=ca, c0_1=cb, phi=out[0],
         q1=out[1], q4=out[2], c_0=out[3], c_1=out[4])
    ncgpu_multicomponent()
    ncgpu_excess()
    ncgpu_new()
    ncgpu_cooling()

    dx = 4.6e-8
    prm = dict(restate.WARREN_DEFAULTS)
    for name, shape, center, r, bc, steps, alpha, seed in [
        ("warren_2d_neumann", (32, 32), (16, 16), 5, "NEUMANN", 10, 0.0, 0),
        # half-integer centres: no cell sits exactly on the seed's centre of
        # symmetry or on the ridge between the seed and its periodic image,
        # where grad(phi) = 0 and the angle arctan2(phi_y, phi_x) is set by
        # rounding residue alone
        ("warren_2d_periodic_noise", (24, 28), (11.5, 13.5), 4, "PERIODIC", 4, 0.3, 7),
        ("warren_2d_mixed_edge", (20, 16), (2, 7.5), 5, ["NEUMANN", "PERIODIC"], 5, 0.0, 0),
    ]:
        phi0 = disk_seed(shape, center, r)
        c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
        p = dict(prm, alpha=alpha)
        noise = [noise_uniform(seed, s, shape) for s in range(steps)] if alpha else None
        phi, c = refshim.run_warren(phi0, c0, steps, bc, dx, p, noise=noise)
        meta = dict(model="warren1995", steps=steps, bc=bc, dx=dx, seed=seed, params=p)
        save(name, meta, phi0=phi0, c0=c0, phi=phi, c=c)


def pseudo_element_tdb(tdb, names, path):
    """A synthetic ideal database with more components: the ternary's records
    plus pseudo-elements `names`, each a copy of Cu's records with its Gibbs
    energies shifted by a few hundred J/mol and its melting point, surface
    energy and kinetic coefficient scaled (no real element's data)."""
    for j, name in enumerate(names):
        shift = 300.0 * (j + 1)
        for phase, fn in (("FCC_A1", "G_CU_FCC"), ("LIQUID", "G_CU_LIQUID")):
            new = "G_" + name + fn[4:]
            tdb.functions[new] = [(lo, hi, f"{expr}+{shift!r}-{0.05 * (j + 1)!r}*T")
                                  for lo, hi, expr in tdb.functions[fn]]
            tdb.params[(phase, name)] = [(298.15, 6000.0, new)]
        for key, scale in (("_L", 1.0 + 0.1 * j), ("_TM", 1.0 - 0.03 * (j + 1)),
                           ("_S", 1.0 + 0.05 * j), ("_B", 1.0 - 0.04 * j)):
            lo, hi, expr = tdb.functions["CU" + key][0]
            tdb.functions[name + key] = [(lo, hi, repr(float(expr) * scale))]
        tdb.elements.append(name)
    tdb.elements.sort()
    write_tdb(tdb, path)


def ncgpu_multicomponent():
    """NCGPU with four and six components (three and five concentration
    fields): the reference's kernels on pseudo-element extensions of
    tests/Ni-Cu-Al_Ideal.tdb."""
    from oracle import ncgpu_ref
    base = refshim.reference_root() / "pyphasefield" / "tests" / "Ni-Cu-Al_Ideal.tdb"
    nrng = np.random.default_rng(20240607)
    for name, extra, shape, c0, seed in [
            ("ncgpu_quaternary", ["XA"], (16, 18), [0.05, 0.3, 0.4], 9),
            ("ncgpu_senary", ["XA", "XB", "XC"], (14, 16), [0.05, 0.2, 0.3, 0.1, 0.15], 13)]:
        tdb_name = f"ncgpu_{len(extra) + 3}comp.tdb"
        pseudo_element_tdb(ncgpu_ref.Tdb(base), extra, HERE / tdb_name)
        tdb = ncgpu_ref.Tdb(HERE / tdb_name)
        p = ncgpu_ref.tdb_params(tdb, 4.6e-6)
        ncomp = len(tdb.elements)
        init = ncgpu_ref.seed_fields(shape, c0=c0, ncomp=ncomp)
        cs = [c + nrng.uniform(-1e-3, 1e-3, shape) for c in init[3:]]
        T = np.full(shape, 1574.0)
        noise = [ncgpu_ref.noise_normal(seed, s, shape) for s in range(3)]
        out = refshim.run_ncgpu(*init[:3], cs, T, 3, p, tdb, noise, "PERIODIC")
        meta = dict(model="ncgpu", steps=3, bc="PERIODIC", seed=seed, dx=4.6e-6, T=1574.0,
                    tdb=tdb_name, ncomp=ncomp)
        arrays = dict(phi0=init[0], q10=init[1], q40=init[2], phi=out[0], q1=out[1], q4=out[2])
        for j, c in enumerate(cs):
            arrays[f"c0_{j}"] = c
            arrays[f"c_{j}"] = out[3 + j]
        save(name, meta, **arrays)


def ncgpu_excess():
    """NCGPU on the reference's non-ideal Ni-Nb database
    (tests/Ni-Nb_Simplified.tdb: binary Redlich-Kister L parameters of
    orders 0-2 in both phases), re-emitted as tests/golden/ncgpu_ninb.tdb."""
    from oracle import ncgpu_ref
    src = refshim.reference_root() / "pyphasefield" / "tests" / "Ni-Nb_Simplified.tdb"
    write_tdb(ncgpu_ref.Tdb(src), HERE / "ncgpu_ninb.tdb")
    tdb = ncgpu_ref.Tdb(HERE / "ncgpu_ninb.tdb")
    assert len(tdb.excess) == 5
    nrng = np.random.default_rng(20240611)
    shape, steps, seed, T0 = (20, 18), 3, 21, 1600.0
    p = ncgpu_ref.tdb_params(tdb, 4.6e-6)
    phi0, q10, q40, c0 = ncgpu_ref.seed_fields(shape, c0=0.10)
    c0 = c0 + nrng.uniform(-1e-3, 1e-3, shape)
    T = np.full(shape, T0)
    noise = [ncgpu_ref.noise_normal(seed, s, shape) for s in range(steps)]
    out = refshim.run_ncgpu(phi0, q10, q40, c0, T, steps, p, tdb, noise, "PERIODIC")
    meta = dict(model="ncgpu", steps=steps, bc="PERIODIC", seed=seed, dx=4.6e-6, T=T0,
                tdb="ncgpu_ninb.tdb")
    save("ncgpu_ninb", meta, phi0=phi0, q10=q10, q40=q40, c0=c0, phi=out[0], q1=out[1],
         q4=out[2], c=out[3])


def ncgpu_new():
    """NCGPU_new (Engines/NCGPU_new.py): its kernels run serially under the
    numba stand-in with the oracle's noise streams (per component, phase and
    orientation), binary Ni-Cu periodic and ternary Ni-Cu-Al zero-gradient."""
    from oracle import ncgpu_ref
    nrng = np.random.default_rng(20240613)
    cases = [("ncgpu_new_periodic", "ncgpu_nicu.tdb", (18, 16), "PERIODIC", [0.40831], 4, 31),
             ("ncgpu_new_ternary", "ncgpu_nicual.tdb", (16, 18), "NEUMANN", [0.05, 0.4], 3, 37)]
    for name, tdb_name, shape, bc, c0, steps, seed in cases:
        tdb = ncgpu_ref.Tdb(HERE / tdb_name)
        p = ncgpu_ref.tdb_params(tdb, 4.6e-6, variant="NCGPU_new")
        init = ncgpu_ref.seed_fields(shape, melt_angle=0.1, seed_angle=0.5, c0=c0,
                                     ncomp=len(tdb.elements))
        cs = [c + nrng.uniform(-1e-3, 1e-3, shape) for c in init[3:]]
        T = np.full(shape, 1574.0)
        noise = [ncgpu_ref.noise_new(seed, s, shape, len(cs)) for s in range(steps)]
        out = refshim.run_ncgpu_new(*init[:3], cs, T, steps, p, tdb, noise, bc)
        meta = dict(model="ncgpu_new", steps=steps, bc=bc, seed=seed, dx=4.6e-6, T=1574.0,
                    tdb=tdb_name)
        arrays = dict(phi0=init[0], q10=init[1], q40=init[2], phi=out[0], q1=out[1], q4=out[2])
        for j, c in enumerate(cs):
            arrays[f"c0_{j}"] = c
            arrays[f"c_{j}"] = out[3 + j]
        save(name, meta, **arrays)


def ncgpu_cooling():
    """NCGPU (Engines/NCGPU.py) under a LINEAR_GRADIENT temperature that also
    changes in time: 2 K per cell along x and -5 K per step (dTdt * dt), the
    reference's kernels run serially with the temperature raised after every
    step as update_thermal_gradient_2D_kernel (ppf_gpu_utils.py:326-334)
    does; no-flux boundaries, Ni-Cu ideal database."""
    os.environ.setdefault("PPF_REFERENCE_ROOT", "/root/reference/pyphasefield")
    from oracle import ncgpu_ref
    tdb = ncgpu_ref.Tdb(HERE / "ncgpu_nicu.tdb")
    shape, steps, seed = (22, 20), 4, 13
    p = ncgpu_ref.tdb_params(tdb, 4.6e-6)
    phi0, q10, q40, c0 = ncgpu_ref.seed_fields(shape, melt_angle=0.1, seed_angle=0.4,
                                               c0=0.40831)
    c0 = c0 + np.random.default_rng(20240606).uniform(-1e-3, 1e-3, shape)
    T = 1576.0 + 2.0 * np.arange(shape[1])[None, :] * np.ones(shape)
    dT_step = -5.0
    noise = [ncgpu_ref.noise_normal(seed, s, shape) for s in range(steps)]
    out = refshim.run_ncgpu(phi0, q10, q40, c0, T, steps, p, tdb, noise, "NEUMANN",
                            dT_step=dT_step)
    meta = dict(model="ncgpu", steps=steps, bc="NEUMANN", seed=seed, dx=4.6e-6, T=1576.0,
                dTdx_per_cell=2.0, dT_step=dT_step, dt=p["dt"], tdb="ncgpu_nicu.tdb")
    save("ncgpu_cooling", meta, phi0=phi0, q10=q10, q40=q40, c0=c0, T0=T, phi=out[0], q1=out[1],
         q4=out[2], c=out[3])


def phase_indefinite():
    """engine_CahnAllenImplicit2D_GMRES (CahnAllen.py:163-175) beyond the
    diagonal-dominance bound: 16 W M dt = 7.28 >= 4 with half the cells at
    phi = 0.75 (the double well's most negative slope), so the system is
    indefinite (90 of 168 eigenvalues negative) yet well conditioned
    (|eigenvalue| >= 0.5), and the reference's GMRES (rtol 1e-5) converges.
    One step: beyond it the next system inherits the indefinite step's
    overshoot."""
    os.environ.setdefault("PPF_REFERENCE_ROOT", "/root/reference/pyphasefield")
    prng = np.random.default_rng(0)
    ud = dict(M=0.7, W=1.3, epsilon=1.1)
    c0 = np.where(prng.random((14, 12)) > 0.5, 0.75, 0.2) + 0.01 * (prng.random((14, 12)) - 0.5)
    fn = "engine_CahnAllenImplicit2D_GMRES"
    dt, dx_ = 0.5, 3.0
    out = refshim.run_implicit(fn, c0, 1, None, dt, dx_, module="CahnAllen", user_data=ud)
    meta = dict(model="allen_cahn", function=fn, steps=1, dt=dt, dx=dx_, solver="implicit",
                adi=False, gmres=True, params=ud)
    save("phase_implicit_ac_2d_gmres_indefinite", meta, c0=c0, out=out)


if __name__ == "__main__":
    if sys.argv[1:] == ["phase_indefinite"]:
        phase_indefinite()
    elif sys.argv[1:] == ["ncgpu_cooling"]:
        ncgpu_cooling()
    elif sys.argv[1:] == ["ncgpu_multicomponent"]:
        ncgpu_multicomponent()
    elif sys.argv[1:] == ["ncgpu_excess"]:
        ncgpu_excess()
    elif sys.argv[1:] == ["ncgpu_new"]:
        ncgpu_new()
    else:
        main()
