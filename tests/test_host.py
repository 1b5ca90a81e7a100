"""Host-side logic without a GPU: the Simulation interface, ghost fill,
checkpoints, boundary structs, the ensemble's thermodynamics and
partitioning, the autotune cache and the C-ABI library's exports."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import restate

ROOT = Path(__file__).resolve().parents[1]


def test_user_data_is_copied_and_defaults_do_not_leak():
    from pyphasefield_gb300 import Warren1995GB300, DiffusionGB300
    shared = {}
    a = DiffusionGB300(dimensions=[8, 8], dx=1.0, dt=0.1, boundary_conditions="PERIODIC",
                       user_data=shared)
    b = Warren1995GB300(dimensions=[8, 8], dx=1.0, boundary_conditions="PERIODIC",
                        user_data=shared)
    assert shared == {}
    assert "T_mA" not in a.user_data and a.user_data["D"] == 0.1
    assert b.user_data["T_mA"] == 1728.0 and "D" not in b.user_data


@pytest.mark.parametrize("bc", ["PERIODIC", "NEUMANN", "DIRCHLET", ["PERIODIC", "NEUMANN"],
                                ["NEUMANN", "DIRCHLET", "PERIODIC"]])
def test_host_ghost_fill_matches_oracle(bc):
    from pyphasefield_gb300 import Simulation
    rng = np.random.default_rng(1)
    nd = 2 if isinstance(bc, str) else len(bc)
    shape = [5, 6, 7][:nd]
    sim = Simulation(dimensions=shape, dx=0.5, boundary_conditions=bc)
    sim.add_field(rng.random(shape), "a")
    sim.add_field(rng.random(shape), "b")
    sim.init_boundary_conditions()
    bcs = [bc] * nd if isinstance(bc, str) else bc
    vals = [[[0.1 * (j + 1), -0.2 * (a + 1)] for a in range(nd)] for j in range(2)]
    for j in range(2):
        for a in range(nd):
            for side, k in ((0, 0), (1, -1)):
                idx = (slice(None),) * a + (k,)
                sim._boundary_conditions_array[j][idx] = vals[j][a][side]
    ref = [f.data.copy() for f in sim.fields]
    sim.apply_boundary_conditions()
    restate.fill_ghosts(ref, bcs, 0.5, vals)
    for f, r in zip(sim.fields, ref):
        np.testing.assert_array_equal(f.data, r)


def test_save_load_round_trip(tmp_path):
    from pyphasefield_gb300 import Simulation
    sim = Simulation(dimensions=[4, 5], save_path=str(tmp_path), boundary_conditions="PERIODIC")
    sim.add_field(np.arange(20.0).reshape(4, 5), "phi")
    sim.add_field(np.ones((4, 5)), "c")
    sim.time_step_counter = 12
    sim.save_simulation()
    other = Simulation(dimensions=None, save_path=str(tmp_path))
    other.load_simulation(step=12)
    assert other.time_step_counter == 12 and other.dimensions == [4, 5]
    np.testing.assert_array_equal(other.fields[0].get_cells(), sim.fields[0].get_cells())
    assert [f.name for f in other.fields] == ["phi", "c"]


def test_begun_simulation_runs_setup_once():
    from pyphasefield_gb300 import Simulation

    class Counting(Simulation):
        calls = 0

        def just_before_simulating(self):
            Counting.calls += 1

    s = Counting(dimensions=[4], boundary_conditions="PERIODIC")
    s.simulate(2)
    s.simulate(3)
    assert Counting.calls == 1 and s.time_step_counter == 5


def test_make_engines_builds_every_engine_on_a_given_base():
    from pyphasefield_gb300 import Simulation, make_engines

    class Host(Simulation):
        pass

    eng = make_engines(Host)
    assert sorted(eng) == ["AllenCahnGB300", "CahnAllenGB300", "CahnHilliardGB300",
                           "DiffusionGB300", "NCGPUGB300", "NCGPU_newGB300", "Warren1995GB300"]
    assert eng["AllenCahnGB300"] is eng["CahnAllenGB300"]
    for cls in eng.values():
        assert issubclass(cls, Host)


def test_warren_rows_per_warp_default():
    """Float Warren1995 engines take eight rows per warp band from 2^22 cells
    up and two below; an explicit tile (the user's or the autotuner's) and
    float64 keep the library default or the given rows."""
    from types import SimpleNamespace

    from pyphasefield_gb300 import Warren1995GB300

    def rows(cells, **ud):
        sim = Warren1995GB300(dimensions=[8, 8], dx=4.6e-8, user_data=ud)
        sim._ppf_grid = SimpleNamespace(cells=cells)
        return sim._ppf_tiling(1).tile_y

    assert rows(1024 * 1024) == 2
    assert rows((1 << 22) - 1) == 2
    assert rows(2048 * 2048) == 8
    assert rows(4096 * 4096) == 8
    assert rows(4096 * 4096, tile=(0, 4)) == 4
    assert rows(4096 * 4096, precision="fp64") == 0


def test_boundary_struct_from_simulation():
    from pyphasefield_gb300 import DiffusionGB300
    from pyphasefield_gb300.device import DeviceGrid, boundary_struct
    import torch
    sim = DiffusionGB300(dimensions=[6, 7], dx=1.0, dt=0.1,
                         boundary_conditions=["DIRCHLET", "NEUMANN"])
    sim.initialize_fields_and_imported_data()
    sim._boundary_conditions_array[0][0, 1:-1] = 0.25
    sim._boundary_conditions_array[0][1:-1, -1] = -1.5
    b = boundary_struct(sim, DeviceGrid([6, 7], torch.float32, torch.device("cpu")), 1)
    assert list(b.type) == [2, 1, 0]
    assert b.value[0][0][0] == 0.25 and b.value[0][1][1] == -1.5
    one = DiffusionGB300(dimensions=[9], dx=1.0, dt=0.1, boundary_conditions="NEUMANN")
    one.initialize_fields_and_imported_data()
    b1 = boundary_struct(one, DeviceGrid([9], torch.float32, torch.device("cpu")), 1)
    assert list(b1.type)[:2] == [0, 1]


def test_warren_liquidus_is_the_equilibrium_liquid():
    from pyphasefield_gb300.ensemble import warren_liquidus
    from pyphasefield_gb300 import Warren1995GB300
    ud = Warren1995GB300.DEFAULTS
    t = warren_liquidus(0.40783, ud)
    assert ud["T_mB"] < t < ud["T_mA"]
    vr = ud["v_m"] / ud["R"]
    ka = np.exp(vr * ud["L_A"] * (1 / t - 1 / ud["T_mA"]))
    kb = np.exp(vr * ud["L_B"] * (1 / t - 1 / ud["T_mB"]))
    assert abs((1 - ka) / (kb - ka) - 0.40783) < 1e-9
    assert warren_liquidus(0.3, ud) > t > warren_liquidus(0.5, ud)


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    from pyphasefield_gb300 import autotune
    monkeypatch.setenv("PPF_AUTOTUNE_CACHE", str(tmp_path / "t.json"))
    calls = []

    def measure(c):
        calls.append(c)
        return {1: 3.0, 2: 1.0, 4: 2.0}[c["d"]]

    cands = [{"d": 1}, {"d": 2}, {"d": 4}]
    assert autotune.pick("k", cands, measure) == {"d": 2}
    assert autotune.pick("k", cands, measure) == {"d": 2}
    assert len(calls) == 3


def _header_functions():
    text = (ROOT / "include" / "ppf_gb300.h").read_text()
    return sorted(set(re.findall(r"^int32_t\s+(ppf_\w+)\s*\(", text, re.M)))


def test_library_exports_every_header_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    names = _header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    from pyphasefield_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == names


def test_library_rejects_bad_arguments_without_gpu(built_lib):
    from pyphasefield_gb300 import _lib as L
    L.load()
    abi, text = L.version()
    assert abi == L.PPF_ABI_VERSION == 3 and "sm_103a" in text
    g = L.PpfGrid()
    g.ndim = 2
    g.shape[0], g.shape[1] = 8, 8
    g.pitch = 6  # < nx
    b = L.PpfBoundary()
    p = L.PpfDiffusionParams(1.0, 0.1, 1.0)
    rc = L.load().ppf_diffusion_step_f32(C.byref(p), C.byref(g), C.byref(b), None, None, None,
                                         None)
    assert rc == L.PPF_ERR_INVALID
    assert "pitch" in L.last_error()
    with pytest.raises(L.PpfError):
        L.call("ppf_diffusion_step_f32", None, C.byref(g), C.byref(b), None, None, None, None)


def test_ensemble_run_validates_without_gpu(built_lib):
    """ppf_ensemble_run_f32 checks its arguments on the host before any
    launch: a NULL plan, a parity other than 0/1, no steps, and (four- and
    eight-row plans) a grid-barrier buffer that is not 8-byte aligned."""
    from pyphasefield_gb300 import _lib as L
    lib = L.load()
    plan = L.PpfEnsemblePlan()
    plan.device_table = 0x1000  # never dereferenced by the host checks
    plan.n_items, plan.n_members, plan.rows, plan.n_units, plan.bands = 4, 1, 4, 1, 1
    t = L.PpfTiling()

    def run(pl, parity=0, nsteps=2, sync=None):
        return lib.ppf_ensemble_run_f32(pl, parity, C.c_uint64(0), None, nsteps,
                                        C.c_void_p(sync) if sync else None, C.byref(t), None)

    assert run(None) == L.PPF_ERR_INVALID
    assert run(C.byref(plan), parity=2) == L.PPF_ERR_INVALID
    assert run(C.byref(plan), nsteps=0) == L.PPF_ERR_INVALID
    assert run(C.byref(plan), sync=0x2004) == L.PPF_ERR_INVALID
    assert "aligned" in L.last_error()


def test_ncgpu_entry_points_validate_without_gpu(built_lib):
    """NCGPU parameter checks run on the host before any launch: component
    count, interaction-term count and indices, NULL buffers."""
    from pyphasefield_gb300 import _lib as L
    lib = L.load()
    g = L.PpfGrid()
    g.ndim = 2
    g.shape[0], g.shape[1] = 8, 8
    g.pitch = 8
    p = L.PpfNcgpuParams()
    p.dx = 1e-4
    dummy = C.c_void_p(16)  # never dereferenced: every call fails validation first
    p.ncomp = 7
    assert lib.ppf_ncgpu_tables_f64(C.byref(p), C.byref(g), dummy, dummy, None) == \
        L.PPF_ERR_UNSUPPORTED
    assert "components" in L.last_error()
    p.ncomp = 2
    p.nexcess = L.PPF_NCGPU_MAX_EXCESS + 1
    assert lib.ppf_ncgpu_tables_f64(C.byref(p), C.byref(g), dummy, dummy, None) == \
        L.PPF_ERR_INVALID
    assert "nexcess" in L.last_error()
    p.nexcess = 1
    p.excess[0].a, p.excess[0].b = 0, 2  # b beyond ncomp
    assert lib.ppf_ncgpu_tables_f64(C.byref(p), C.byref(g), dummy, dummy, None) == \
        L.PPF_ERR_INVALID
    assert "excess term 0" in L.last_error()
    assert lib.ppf_ncgpu_tables_f64(C.byref(p), C.byref(g), None, dummy, None) == \
        L.PPF_ERR_INVALID


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct of include/ppf_gb300.h has the same size and field
    offsets in the ctypes binding as gcc lays it out (a layout mismatch
    would pass garbage across the ABI without an error)."""
    import shutil
    import subprocess
    from pyphasefield_gb300 import _lib as L
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = [n for n in dir(L) if n.startswith("Ppf") and isinstance(getattr(L, n), type)
               and issubclass(getattr(L, n), C.Structure)]
    assert len(structs) >= 14
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ppf_gb300.h"',
             "int main(void) {"]
    for n in structs:
        lines.append(f'  printf("{n} size %zu\\n", sizeof({n}));')
        for fname, _ in getattr(L, n)._fields_:
            lines.append(f'  printf("{n} {fname} %zu\\n", offsetof({n}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    seen = 0
    for line in out.splitlines():
        n, field, value = line.split()
        cls = getattr(L, n)
        expect = C.sizeof(cls) if field == "size" else getattr(cls, field).offset
        assert int(value) == expect, (n, field, int(value), expect)
        seen += 1
    assert seen > len(structs)


def test_ctypes_signatures_match_the_header_argument_counts():
    """Each entry point's ctypes argtypes has as many arguments as its C
    prototype in include/ppf_gb300.h."""
    from pyphasefield_gb300 import _lib as L
    text = (ROOT / "include" / "ppf_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = dict(re.findall(r"int32_t\s+(ppf_\w+)\s*\(([^)]*)\)\s*;", text))
    assert sorted(protos) == sorted(L.SIGNATURES)
    for name, args in protos.items():
        args = args.strip()
        n = 0 if args in ("", "void") else args.count(",") + 1
        assert len(L.SIGNATURES[name]) == n, (name, n, len(L.SIGNATURES[name]))


def test_header_constants_match_the_binding():
    """Every #define of include/ppf_gb300.h that the ctypes binding also
    names has the same value there."""
    from pyphasefield_gb300 import _lib as L
    text = (ROOT / "include" / "ppf_gb300.h").read_text()
    defines = dict(re.findall(r"^#define\s+(PPF_\w+)\s+\(?(-?\d+)\)?", text, re.M))
    shared = [n for n in defines if hasattr(L, n)]
    assert len(shared) >= 10
    for n in shared:
        assert getattr(L, n) == int(defines[n]), n
