"""Filter interface (sktopt/filters/base.py:9-37)."""
from __future__ import annotations

import numpy as np


class BaseFilter:
    def __init__(self, mesh, elements_volume, radius, design_mask=None):
        self.mesh = mesh
        self.elements_volume = np.asarray(elements_volume, dtype=np.float64)
        self.radius = radius
        self.design_mask = None if design_mask is None else np.asarray(design_mask, bool)

    def update_radius(self, radius, **args):
        raise NotImplementedError("")

    @classmethod
    def from_defaults(cls, mesh, elements_volume, radius=0.3, design_mask=None):
        raise NotImplementedError("")

    def forward(self, rho_element):
        raise NotImplementedError("")

    def gradient(self, v):
        raise NotImplementedError("")
