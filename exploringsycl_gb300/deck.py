"""tea.in decks: writer, the standard layouts, and the seeded random-state
generator.

The deck grammar is the reference's (TeaLeaf/parse_config.c:77-286): one
``key=value`` or ``key value`` per line, states as
``state N density=.. energy=.. geometry=rectangle|circular|point xmin=..
xmax=.. ymin=.. ymax=.. [radius=..]``. Circular states must still carry
xmax/ymax because the parser reads them unconditionally
(parse_config.c:257-260); the parser takes a disc's centre from xmin/ymin.
Values are written with full double precision.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path


@dataclass
class State:
    density: float
    energy: float
    geometry: str = "rectangle"      # rectangle | circular | point
    xmin: float = 0.0
    xmax: float = 0.0
    ymin: float = 0.0
    ymax: float = 0.0
    radius: float = 0.0


@dataclass
class Deck:
    x_cells: int
    y_cells: int
    states: list[State]
    end_step: int = 10
    max_iters: int = 10000
    eps: float = 1.0e-15
    initial_timestep: float = 0.004
    xmin: float = 0.0
    ymin: float = 0.0
    xmax: float = 10.0
    ymax: float = 10.0
    solver: str = "cg"              # cg | jacobi | chebyshev | ppcg
    halo_depth: int | None = None
    summary_frequency: int | None = None
    presteps: int | None = None
    ppcg_inner_steps: int | None = None
    coefficient: str | None = None  # density | inverse_density
    extra: list[str] = field(default_factory=list)

    def text(self) -> str:
        out = ["*tea"]
        for n, s in enumerate(self.states, start=1):
            line = f"state {n} density={s.density!r} energy={s.energy!r}"
            if n > 1:
                line += f" geometry={s.geometry} xmin={s.xmin!r} xmax={s.xmax!r}"
                line += f" ymin={s.ymin!r} ymax={s.ymax!r}"
                if s.geometry == "circular":
                    line += f" radius={s.radius!r}"
            out.append(line)
        out += [f"x_cells={self.x_cells}", f"y_cells={self.y_cells}",
                f"xmin={self.xmin!r}", f"ymin={self.ymin!r}", f"xmax={self.xmax!r}",
                f"ymax={self.ymax!r}", f"initial_timestep={self.initial_timestep!r}",
                f"end_step={self.end_step}", f"max_iters={self.max_iters}",
                f"use_{self.solver}", f"eps {self.eps!r}"]
        if self.halo_depth is not None:
            out.append(f"halo_depth={self.halo_depth}")
        if self.summary_frequency is not None:
            out.append(f"summary_frequency={self.summary_frequency}")
        if self.presteps is not None:
            out.append(f"presteps={self.presteps}")
        if self.ppcg_inner_steps is not None:
            out.append(f"ppcg_inner_steps={self.ppcg_inner_steps}")
        if self.coefficient is not None:
            out.append(f"coefficient_{self.coefficient}")
        out += list(self.extra)
        out.append("*endtea")
        return "\n".join(out) + "\n"

    def write(self, path: str | Path) -> Path:
        p = Path(path)
        p.write_text(self.text())
        return p


def five_state(n: int, end_step: int = 10, **kw) -> Deck:
    """The standard TeaLeaf deck of tea.in and the benchmark decks: a
    background of density 100 / energy 1e-4 and four thin hot rectangles."""
    states = [
        State(100.0, 0.0001),
        State(0.1, 25.0, "rectangle", 0.0, 1.0, 1.0, 2.0),
        State(0.1, 0.1, "rectangle", 1.0, 6.0, 1.0, 2.0),
        State(0.1, 0.1, "rectangle", 5.0, 6.0, 1.0, 8.0),
        State(0.1, 0.1, "rectangle", 5.0, 10.0, 7.0, 8.0),
    ]
    return Deck(n, n, states, end_step=end_step, **kw)


def two_state(n: int, end_step: int = 10, **kw) -> Deck:
    """Background density 100 / energy 1e-4 with one hot rectangle
    x in [0,1], y in [1,2] at density 0.1 / energy 25."""
    states = [State(100.0, 0.0001), State(0.1, 25.0, "rectangle", 0.0, 1.0, 1.0, 2.0)]
    return Deck(n, n, states, end_step=end_step, **kw)


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood, 2014): the same stream in C and Python."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.state = seed & self.MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        """Uniform double in [0, 1) with 53 random bits."""
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))


def random_states(seed: int, extent: float = 10.0, min_shapes: int = 20,
                  max_shapes: int = 60, density_range=(0.05, 200.0),
                  energy_range=(1e-4, 25.0)) -> list[State]:
    """Seeded random piecewise-constant layout: a background state, then
    20-60 axis-aligned rectangles and discs, density log-uniform and energy
    uniform in the given ranges. Coordinates are rounded to 1e-6 so that
    the deck text reproduces them exactly."""
    rng = SplitMix64(seed)
    lo, hi = math.log(density_range[0]), math.log(density_range[1])

    def dens() -> float:
        return round(math.exp(lo + (hi - lo) * rng.uniform()), 9)

    def ener() -> float:
        return round(energy_range[0] + (energy_range[1] - energy_range[0]) * rng.uniform(), 9)

    states = [State(dens(), ener())]
    n = min_shapes + int(rng.uniform() * (max_shapes - min_shapes + 1))
    for _ in range(n):
        if rng.uniform() < 0.5:
            w = extent * (0.02 + 0.25 * rng.uniform())
            h = extent * (0.02 + 0.25 * rng.uniform())
            x0 = (extent - w) * rng.uniform()
            y0 = (extent - h) * rng.uniform()
            states.append(State(dens(), ener(), "rectangle", round(x0, 6), round(x0 + w, 6),
                                round(y0, 6), round(y0 + h, 6)))
        else:
            r = extent * (0.01 + 0.12 * rng.uniform())
            cx = extent * rng.uniform()
            cy = extent * rng.uniform()
            states.append(State(dens(), ener(), "circular", round(cx, 6), round(cx + r, 6),
                                round(cy, 6), round(cy + r, 6), round(r, 6)))
    return states


def random_deck(n: int, seed: int, end_step: int = 1, **kw) -> Deck:
    return Deck(n, n, random_states(seed), end_step=end_step, **kw)
