"""Beamline container with the reference's sorting and lookup behaviour.

Mirrors ``src/trajectories/beamline.py``: elements are sorted by ``z0`` once at
construction (stable ``list.sort``, :17-18,40-45) and ``find_element`` returns
the first element with a matching name or prints and returns None (:47-55).
``propagate_through`` has no Python body here: molecules are propagated on the
GPU by :class:`ctraj.trajectory_simulator.TrajectorySimulator`.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

__all__ = ["Beamline"]


@dataclass
class Beamline:
    elements: List

    def __post_init__(self):
        self.sort_elements()

    def sort_elements(self):
        self.elements.sort(key=lambda e: e.z0)

    def save_to_hdf(self, filepath, run_name: str) -> None:
        """beamline.py:78-90: one group per element under run_name/beamline."""
        from .hdf import save_beamline

        save_beamline(self, filepath, run_name)

    def find_element(self, name):
        for element in self.elements:
            if element.name == name:
                return element
        print(f"Element with name '{name}' not found in beamline")
