"""Simulation base class with the reference's plugin interface
(pyphasefield simulation.py:19-723): the same constructor keywords, lifecycle
hooks, getters/setters, ghost-cell fill and .npz checkpoint format, so that
engine subclasses written against pyphasefield run unchanged.

Differences from the reference, each a defect corrected:
  * ``user_data`` is copied per instance (the reference's default ``{}`` is
    shared by every instance, simulation.py:25, so engine defaults leak).
  * ``simulate`` sets ``_begun_simulation = True`` (the reference compares
    with ``==`` at simulation.py:260 and re-runs just_before_simulating on
    every call).
  * ``just_before_simulating`` checks the temperature shape only when a
    temperature field exists (simulation.py:289 asserts unconditionally).
  * ``apply_boundary_conditions`` fills the ghosts of every axis (the
    reference's slices for axes >= 1 at simulation.py:561-566 index a new
    axis and never fill them).
  * ``load_simulation`` falls back to step 0 when the file name has no
    ``step_N`` (the reference's check at :381 can never trigger).
Out of this package's scope (they raise): XDMF thermal files (meshio),
CALPHAD databases (pycalphad) and plotting (matplotlib).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .field import Field

BC_TYPES = ("PERIODIC", "NEUMANN", "DIRCHLET")


def bc_per_axis(sim, nd: int) -> list[str]:
    """Per-axis boundary types from Simulation._boundary_conditions_type
    (one string for every axis, or a list with one string per axis)."""
    bc = sim._boundary_conditions_type
    if bc is None:
        raise ValueError("boundary_conditions must be set (PERIODIC, NEUMANN or DIRCHLET)")
    bcs = [bc] * nd if isinstance(bc, str) else list(bc)
    if len(bcs) != nd or any(b not in BC_TYPES for b in bcs):
        raise ValueError(f"boundary_conditions {bc!r} invalid for {nd} dimensions")
    return bcs


def fill_ghosts_host(sim) -> None:
    """Ghost fill of the host copies (Field.data) of every field, axis by
    axis in the reference's order, filling every axis: PERIODIC wraps,
    NEUMANN sets ghost = edge -/+ dx*value, DIRCHLET sets ghost = value, with
    values from _boundary_conditions_array. The temperature field gets
    periodic ghosts on periodic axes and zero-gradient ghosts otherwise."""
    if not sim.fields:
        return
    nd = sim.fields[0].data.ndim
    bcs = bc_per_axis(sim, nd)
    arr = sim._boundary_conditions_array
    if arr is None:
        arr = np.zeros([len(sim.fields)] + list(sim.fields[0].data.shape))

    def at(axis, k):
        return (slice(None),) * axis + (k,)

    for i, b in enumerate(bcs):
        if sim.temperature is not None:
            t = sim.temperature.data
            if b == "PERIODIC":
                t[at(i, 0)] = t[at(i, -2)]
                t[at(i, -1)] = t[at(i, 1)]
            else:
                t[at(i, 0)] = t[at(i, 1)]
                t[at(i, -1)] = t[at(i, -2)]
        for j, f in enumerate(sim.fields):
            d = f.data
            if b == "PERIODIC":
                d[at(i, 0)] = d[at(i, -2)]
                d[at(i, -1)] = d[at(i, 1)]
            elif b == "NEUMANN":
                d[at(i, 0)] = d[at(i, 1)] - sim.dx * arr[j][at(i, 0)]
                d[at(i, -1)] = d[at(i, -2)] + sim.dx * arr[j][at(i, -1)]
            else:
                d[at(i, 0)] = arr[j][at(i, 0)]
                d[at(i, -1)] = arr[j][at(i, -1)]


class Simulation:
    def __init__(self, dimensions, framework=None, dx=None, dt=None, initial_time_step=0,
                 temperature_type=None, initial_T=None, dTdx=None, dTdy=None, dTdz=None,
                 dTdt=None, temperature_path=None, temperature_units="K",
                 tdb_container=None, tdb_path=None, tdb_components=None, tdb_phases=None,
                 save_path=None, autosave=False, save_images=False, autosave_rate=None,
                 boundary_conditions=None, user_data=None):
        self._framework = framework
        self._uses_gpu = False
        self._begun_simulation = False

        self.fields: list[Field] = []
        self.dimensions = list(dimensions) if dimensions is not None else None
        self.dx = dx
        self.dt = dt
        self.time_step_counter = initial_time_step

        self.temperature = None
        self._temperature_type = temperature_type
        self._temperature_path = temperature_path
        self._temperature_units = temperature_units
        self._initial_T = initial_T
        self._dTdx, self._dTdy, self._dTdz, self._dTdt = dTdx, dTdy, dTdz, dTdt

        self._tdb_container = tdb_container
        self._tdb_path = tdb_path
        self._tdb_components = tdb_components
        self._tdb_phases = tdb_phases

        self._save_path = save_path
        self._autosave_flag = autosave
        self._autosave_rate = autosave_rate
        self._autosave_save_images_flag = save_images

        self._boundary_conditions_type = boundary_conditions
        self._boundary_conditions_array = None

        self._debug_mode_flag = False
        self.user_data = dict(user_data) if user_data is not None else {}

    # ---------------------------------------------------------------- hooks
    def init_fields(self):
        """Engine subclasses add their fields here (base adds none)."""

    def init_boundary_conditions(self):
        """Zero-filled per-field boundary value array over the padded grid
        (simulation.py:109-123): Neumann gradients / Dirichlet values."""
        dims = [n + 2 for n in self.dimensions]
        self._boundary_conditions_array = np.zeros([len(self.fields)] + dims)

    def init_temperature_field(self):
        t = self._temperature_type
        if t is None:
            return
        if t == "ISOTHERMAL":
            arr = np.full(self.dimensions, float(self._initial_T))
        elif t == "LINEAR_GRADIENT":
            arr = np.full(self.dimensions, float(self._initial_T))
            nd = len(self.dimensions)
            for grad, axis in ((self._dTdx, nd - 1), (self._dTdy, nd - 2), (self._dTdz, nd - 3)):
                if axis < 0 or not grad:
                    continue
                shape = [1] * nd
                shape[axis] = self.dimensions[axis]
                arr = arr + (np.arange(self.dimensions[axis]) * self.dx * grad).reshape(shape)
            arr = arr + self.time_step_counter * (self._dTdt or 0.0)
        elif t == "XDMF_FILE":
            raise NotImplementedError("XDMF thermal histories need meshio, which this "
                                      "package does not use")
        else:
            raise ValueError("Unknown temperature profile.")
        self.temperature = Field(data=arr, simulation=self, colormap="jet",
                                 name=f"Temperature ({self._temperature_units})")

    def init_tdb_params(self):
        if self._tdb_container is not None or self._tdb_path is not None:
            raise NotImplementedError("CALPHAD databases (pycalphad) are outside this package")

    def initialize_fields_and_imported_data(self):
        if self._framework in ("GPU_SERIAL", "GPU_PARALLEL"):
            self._uses_gpu = True
        self.init_tdb_params()
        self.init_temperature_field()
        self.init_fields()
        self.init_boundary_conditions()

    def just_before_simulating(self):
        if self._uses_gpu:
            self.send_fields_to_GPU()
        self.apply_boundary_conditions()
        if self.temperature is not None and self.fields:
            assert self.temperature.data.shape == self.fields[0].data.shape

    def simulation_loop(self):
        """Advance the fields by one step (engines override)."""

    def simulate(self, number_of_timesteps):
        """Per step: counter += 1, simulation_loop, temperature update, ghost
        fill, autosave every _autosave_rate steps (simulation.py:245-271)."""
        if not self._begun_simulation:
            self._begun_simulation = True
            self.just_before_simulating()
        for _ in range(number_of_timesteps):
            self.time_step_counter += 1
            self.simulation_loop()
            self.update_temperature_field()
            self.apply_boundary_conditions()
            if self._autosave_flag and self.time_step_counter % self._autosave_rate == 0:
                if self._uses_gpu:
                    self.retrieve_fields_from_GPU()
                self.save_simulation()

    def add_field(self, array, array_name, colormap="GnBu"):
        self.fields.append(Field(data=array, name=array_name, simulation=self,
                                 colormap=colormap))

    def default_value(self, var, value):
        if getattr(self, var, None) is None:
            setattr(self, var, value)

    def update_temperature_field(self, force_cpu=False):
        t = self._temperature_type
        if t is None or t == "ISOTHERMAL":
            return
        if t == "LINEAR_GRADIENT":
            self.temperature.data += self._dTdt * self.dt
            return
        if t == "XDMF_FILE":
            raise NotImplementedError("XDMF thermal histories need meshio")
        raise ValueError("Unknown temperature profile.")

    # ------------------------------------------------------ boundary fill
    def apply_boundary_conditions(self):
        """Host ghost fill (simulation.py:560-618), axis by axis, every axis."""
        fill_ghosts_host(self)

    def send_fields_to_GPU(self):
        """Engines with a device path override this."""

    def retrieve_fields_from_GPU(self):
        """Engines with a device path override this."""

    # ------------------------------------------------------- checkpoints
    def save_simulation(self, step=None):
        """np.savez of every field's interior, keyed by field name, to
        <save_path>/step_<counter>.npz (simulation.py:399-420); `step`
        overrides the counter in the file name (asynchronous autosave)."""
        if not self._save_path:
            print("self._save_path not defined, aborting save!")
            return
        loc = Path(self._save_path)
        loc.mkdir(parents=True, exist_ok=True)
        n = self.time_step_counter if step is None else int(step)
        np.savez(str(loc) + "/step_" + str(n), **{f.name: f.get_cells() for f in self.fields})
        return 0

    def load_simulation(self, file_path=None, step=-1):
        """Inverse of save_simulation (simulation.py:334-397)."""
        self.fields = []
        if file_path is None:
            file_path = self._save_path
            if self._save_path is None:
                raise ValueError("Simulation needs a path to load data from!")
        if Path.cwd().joinpath(file_path).exists():
            file_path = Path.cwd().joinpath(file_path)
        elif self._save_path is not None and \
                Path.cwd().joinpath(self._save_path).joinpath(file_path).exists():
            file_path = Path.cwd().joinpath(self._save_path).joinpath(file_path)
        else:
            file_path = Path(file_path)
        if file_path.is_dir():
            if step > -1:
                file_path = file_path.joinpath("step_" + str(step) + ".npz")
            else:
                raise ValueError("Given path is a folder, must specify a timestep!")
        if self._save_path is None:
            self._save_path = str(file_path.parent)
        with np.load(file_path, allow_pickle=True) as npz:
            for key in npz.files:
                self.add_field(npz[key], key)
        self.dimensions = list(self.fields[0].get_cells().shape)
        if step < 0:
            name = file_path.stem
            k = name.find("step_")
            if k < 0:
                self.time_step_counter = 0
            else:
                i = j = k + len("step_")
                while j < len(name) and name[j].isdigit():
                    j += 1
                self.time_step_counter = int(name[i:j]) if j > i else 0
        else:
            self.time_step_counter = int(step)
        if self._temperature_type == "LINEAR_GRADIENT" and self.temperature is not None:
            self.temperature.data += self.time_step_counter * self._dTdt * self.dt
        self._begun_simulation = False
        return 0

    # --------------------------------------------------------- plotting
    def plot_simulation(self, *args, **kwargs):
        raise NotImplementedError("plotting (matplotlib) is outside this package; use "
                                  "get_cells() of each field")

    def plot_all_fields(self):
        return self.plot_simulation()

    def plot_field(self, f, save_path=None):
        return self.plot_simulation()

    def progress_bar(self):
        return

    def generate_python_script(self):
        return

    # ------------------------------------------------- getters / setters
    def set_dimensions(self, dimensions):
        self.dimensions = dimensions

    def get_dimensions(self):
        return self.dimensions

    def set_framework(self, framework):
        self._framework = framework

    def get_framework(self):
        return self._framework

    def set_dx(self, dx):
        self.dx = dx

    def set_cell_spacing(self, dx):
        self.dx = dx

    def get_dx(self):
        return self.dx

    def get_cell_spacing(self):
        return self.dx

    def set_dt(self, dt):
        self.dt = dt

    def set_time_step_length(self, dt):
        self.dt = dt

    def get_dt(self):
        return self.dt

    def get_time_step_length(self):
        return self.dt

    def set_time_step_counter(self, time_step_counter):
        self.time_step_counter = time_step_counter

    def get_time_step_counter(self):
        return self.time_step_counter

    def increment_time_step_counter(self):
        self.time_step_counter += 1

    def set_temperature_type(self, temperature_type):
        self._temperature_type = temperature_type

    def set_temperature_initial_T(self, initial_T):
        self._initial_T = initial_T

    def set_temperature_dTdx(self, dTdx):
        self._dTdx = dTdx

    def set_temperature_dTdy(self, dTdy):
        self._dTdy = dTdy

    def set_temperature_dTdz(self, dTdz):
        self._dTdz = dTdz

    def set_temperature_dTdt(self, dTdt):
        self._dTdt = dTdt

    def set_temperature_path(self, temperature_path):
        self._temperature_path = temperature_path

    def set_temperature_units(self, temperature_units):
        self._temperature_units = temperature_units

    def set_tdb_container(self, tdb_container):
        self._tdb_container = tdb_container

    def set_tdb_path(self, tdb_path):
        self._tdb_path = tdb_path

    def set_tdb_phases(self, tdb_phases):
        self._tdb_phases = tdb_phases

    def set_tdb_components(self, tdb_components):
        self._tdb_components = tdb_components

    def set_save_path(self, save_path):
        self._save_path = save_path

    def set_autosave_flag(self, autosave_flag):
        self._autosave_flag = autosave_flag

    def set_autosave_save_images_flag(self, autosave_save_images_flag):
        self._autosave_save_images_flag = autosave_save_images_flag

    def set_autosave_rate(self, autosave_rate):
        self._autosave_rate = autosave_rate

    def set_boundary_conditions(self, boundary_conditions_type):
        self._boundary_conditions_type = boundary_conditions_type

    def set_user_data(self, data):
        self.user_data = data

    def set_debug_mode_flag(self, debug_mode_flag):
        self._debug_mode_flag = debug_mode_flag
