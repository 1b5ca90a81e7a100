"""Host-side Field container with the reference's interface
(pyphasefield field.py:4-73): a float64 array padded by one ghost layer per
side, zero-filled at construction, plus the reference's stencil helpers.

On a GB300 engine the field's authoritative copy lives on the device
(interior only, float32 or float64); ``Field.data`` is refreshed by
``retrieve_fields_from_GPU`` and read by ``send_fields_to_GPU``.
"""
from __future__ import annotations

import numpy as np


class Field:
    def __init__(self, data=None, simulation=None, name=None, colormap="GnBu"):
        data = np.asarray(data, dtype=np.float64)
        self._slice = tuple(slice(1, -1) for _ in range(data.ndim))
        padded = np.zeros([n + 2 for n in data.shape])
        padded[self._slice] += data
        self.data = padded
        self.name = name
        self._simulation = simulation
        self.colormap = colormap

    def __str__(self):
        return str(self.data)

    # --- stencils on the padded array (field.py:26-67) -------------------
    def _inv_dx(self) -> float:
        return 1.0 / self._simulation.get_cell_spacing()

    def gradient_cell(self) -> np.ndarray:
        """Central difference along every axis, stacked on a new axis 0."""
        h = 0.5 * self._inv_dx()
        return np.stack([(np.roll(self.data, -1, a) - np.roll(self.data, 1, a)) * h
                         for a in range(self.data.ndim)])

    def gradient_face_left(self) -> np.ndarray:
        h = self._inv_dx()
        return np.stack([(self.data - np.roll(self.data, 1, a)) * h
                         for a in range(self.data.ndim)])

    def gradient_face_right(self) -> np.ndarray:
        h = self._inv_dx()
        return np.stack([(np.roll(self.data, -1, a) - self.data) * h
                         for a in range(self.data.ndim)])

    def laplacian(self) -> np.ndarray:
        h2 = self._inv_dx() ** 2
        out = (np.roll(self.data, -1, 0) + np.roll(self.data, 1, 0) - 2 * self.data) * h2
        for a in range(1, self.data.ndim):
            out += (np.roll(self.data, -1, a) + np.roll(self.data, 1, a) - 2 * self.data) * h2
        return out

    def get_cells(self) -> np.ndarray:
        return self.data[self._slice]

    def get_all_cells(self) -> np.ndarray:
        return self.data
