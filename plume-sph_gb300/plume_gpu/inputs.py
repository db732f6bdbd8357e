"""Reader of the reference's run-time input files.

`read_data` restates Read_Data (src/plume/dataread.cc:77-245): `scale.data`
holds the length and gravity scales; `simulation.data` is read line by line
in a fixed order, each value taken after the last ':' and converted with
`stof` (so every number passes through single precision before it is stored
as a double, as the reference does).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np


def _stof(text: str) -> float:
    """C++ std::stof then widening to double (dataread.cc:110-200)."""
    return float(np.float32(float(text.strip().split()[0]) if text.strip() else 0.0))


@dataclass
class SimulationData:
    max_time: float
    max_steps: int
    timeoutput: float
    stat_erupt: float
    end_erupt: float
    format: int
    p_constant: float
    gamma: float
    smoothing_length: float
    idom: tuple                 # (x_min, x_max, y_min, y_max, z_min, z_max)
    length_scale: float = 1.0
    gravity_scale: float = 1.0
    meteo: tuple | None = None  # (rows, cols, path) when present


def read_data(directory: str = ".") -> SimulationData:
    """Parse scale.data and simulation.data from `directory`."""
    ls, gs = 1.0, 1.0
    sp = os.path.join(directory, "scale.data")
    if os.path.exists(sp):
        vals = open(sp).read().split()
        if len(vals) >= 2:
            ls, gs = float(vals[0]), float(vals[1])
    path = os.path.join(directory, "simulation.data")
    if not os.path.exists(path):
        raise FileNotFoundError('ERROR: Can\'t find "simulation.data" input file.')
    lines = open(path).read().splitlines()

    def val(i):
        if i >= len(lines):
            raise ValueError(f"simulation.data: missing line {i + 1}")
        return lines[i][lines[i].rfind(":") + 1:]

    f = [_stof(val(i)) for i in range(15)]
    meteo = None
    if len(lines) >= 18:
        meteo = (int(_stof(val(15))), int(_stof(val(16))), val(17).strip())
    return SimulationData(
        max_time=f[0], max_steps=int(f[1]), timeoutput=f[2], stat_erupt=f[3],
        end_erupt=f[4], format=int(f[5]), p_constant=f[6], gamma=f[7],
        smoothing_length=f[8] / ls, idom=tuple(f[9:15]), length_scale=ls,
        gravity_scale=gs, meteo=meteo)


def write_data(directory: str, sim: SimulationData) -> None:
    """Write simulation.data / scale.data in the reference's line order."""
    labels = [
        ("maximum simulation time(s)", sim.max_time),
        ("maximum simulation time step", sim.max_steps),
        ("output time interval(s)", sim.timeoutput),
        ("start eruption time(s)", sim.stat_erupt),
        ("end eruption time(s)", sim.end_erupt),
        ("output format indicator, 0 for matlab readable data, 1 for h5part data", sim.format),
        ("P_CONSTANT, the constant in equation of state for ideal gas", sim.p_constant),
        ("the ratio between specific heat of constant pressure and that of constant volume", sim.gamma),
        ("smoothing length for air particles", sim.smoothing_length * sim.length_scale),
        ("minimun x coordinate of initial domain", sim.idom[0]),
        ("maximum x coordinate of initial domain", sim.idom[1]),
        ("minimun y coordinate of initial domain", sim.idom[2]),
        ("maximum y coordinate of initial domain", sim.idom[3]),
        ("minimum z coordinate of initial domain", sim.idom[4]),
        ("maximum z coordinate of initial domain", sim.idom[5]),
    ]
    with open(os.path.join(directory, "simulation.data"), "w") as fp:
        for lab, v in labels:
            fp.write(f"{lab}:{v!r}\n")
    with open(os.path.join(directory, "scale.data"), "w") as fp:
        fp.write(f"{sim.length_scale}\n{sim.gravity_scale}\n")
