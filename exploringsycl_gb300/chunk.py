"""A TeaLeaf chunk held on the GPU and driven through the C ABI.

``GpuChunk`` performs, from Python, the same sequence of backend calls as
the TeaLeaf driver (TeaLeaf/initialise.c:11-31 for set-up,
TeaLeaf/diffuse.c:23-78 and drivers/cg_driver.c for a timestep), so that
tests and the benchmark can drive the kernels without the C++ driver. One
chunk, external faces on all four sides.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import (CONDUCTIVITY, MAX_CELLS, METHODS, Context, TLError, TLSolveParams,
               TLSolveReport, TLState, check)
from .deck import Deck

GEOMETRY = {"rectangle": 0, "circular": 1, "point": 2}
FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w", "kx",
          "ky", "sd", "volume"]


def parsed_states(deck: Deck) -> list[TLState]:
    """States as the deck parser stores them: bounds moved a hundredth of a
    cell inwards and disc centres moved by the same amount
    (TeaLeaf/parse_config.c:222-260)."""
    dx = (deck.xmax - deck.xmin) / deck.x_cells
    dy = (deck.ymax - deck.ymin) / deck.y_cells
    out = []
    for n, s in enumerate(deck.states):
        t = TLState()
        t.density, t.energy = s.density, s.energy
        if n > 0:
            t.x_min = s.xmin + dx / 100.0
            t.y_min = s.ymin + dy / 100.0
            t.x_max = s.xmax - dx / 100.0
            t.y_max = s.ymax - dy / 100.0
            t.radius = s.radius
            t.geometry = GEOMETRY[s.geometry]
        out.append(t)
    return out


class GpuChunk:
    def __init__(self, deck: Deck, ctx: Context | None = None, device: int = 0):
        self.deck = deck
        self.hd = deck.halo_depth or 2
        self.x = deck.x_cells + 2 * self.hd
        self.y = deck.y_cells + 2 * self.hd
        self.n = self.x * self.y
        if self.n > MAX_CELLS:
            raise TLError(f"grid of {self.x} x {self.y} cells (halos included) exceeds "
                          f"TL_MAX_CELLS ({MAX_CELLS} cells)")
        self.ctx = ctx or Context(device)
        self.dx = (deck.xmax - deck.xmin) / deck.x_cells
        self.dy = (deck.ymax - deck.ymin) / deck.y_cells
        self.coefficient = CONDUCTIVITY if deck.coefficient in (None, "density") else 2
        self.f = {name: self.ctx.alloc(self.n) for name in FIELDS}
        self.f["x_area"] = self.ctx.alloc((self.x + 1) * self.y)
        self.f["y_area"] = self.ctx.alloc(self.x * (self.y + 1))
        for name, n in (("cell_x", self.x), ("cell_y", self.y), ("vertex_x", self.x + 1),
                        ("vertex_y", self.y + 1)):
            self.f[name] = self.ctx.alloc(n)
        self.max_iters = deck.max_iters
        self.pw_hist = np.zeros(max(self.max_iters, 1))
        self.rrn_hist = np.zeros(max(self.max_iters, 1))
        self.last_steps = 0
        self.initialise()

    def call(self, name, *args):
        self.ctx.call(name, *args)

    def halos(self, names: list[str], depth: int) -> None:
        arr = (C.c_void_p * len(names))(*[self.f[n] for n in names])
        self.call("tl_local_halos", self.x, self.y, self.hd, depth, 0xF, arr, len(names))

    def initialise(self) -> None:
        x, y, hd, f = self.x, self.y, self.hd, self.f
        d = self.deck
        self.call("tl_set_chunk_data_vertices", x, y, hd, f["vertex_x"], f["vertex_y"],
                  d.xmin, d.ymin, self.dx, self.dy)
        self.call("tl_set_chunk_data", x, y, hd, f["vertex_x"], f["vertex_y"], f["cell_x"],
                  f["cell_y"], f["volume"], f["x_area"], f["y_area"], d.xmin, d.ymin,
                  self.dx, self.dy)
        states = parsed_states(d)
        self.call("tl_set_chunk_initial_state", x, y, states[0].energy, states[0].density,
                  f["energy0"], f["density"])
        for s in states[1:]:
            self.call("tl_set_chunk_state", x, y, hd, C.byref(s), f["energy0"], f["density"],
                      f["u"], f["cell_x"], f["cell_y"], f["vertex_x"], f["vertex_y"])
        self.halos(["density", "energy0", "energy"], 2)
        self.call("tl_store_energy", x, y, f["energy"], f["energy0"])

    def rx_ry(self) -> tuple[float, float]:
        dt = self.deck.initial_timestep
        return dt / (self.dx * self.dx), dt / (self.dy * self.dy)

    def cg_timestep(self) -> int:
        """One timestep with the device CG solve (the run-ahead path of the
        backend); returns the number of CG steps executed."""
        x, y, hd, f = self.x, self.y, self.hd, self.f
        rx, ry = self.rx_ry()
        self.halos(["energy", "density"], 2)
        rro = C.c_double(0.0)
        steps = C.c_int(0)
        self.call("tl_cg_solve", x, y, hd, self.coefficient, rx, ry, self.deck.eps,
                  self.max_iters, f["p"], f["r"], f["u"], f["u0"], f["w"], f["kx"], f["ky"],
                  f["density"], f["energy"], C.byref(rro),
                  self.pw_hist.ctypes.data_as(C.POINTER(C.c_double)),
                  self.rrn_hist.ctypes.data_as(C.POINTER(C.c_double)), C.byref(steps))
        self.rro0 = rro.value
        self.last_steps = steps.value
        self.solve_finished()
        return steps.value

    def solve_timestep(self, method: str = "mixed", rel_tol: float = 1e-10,
                       inner_tol: float = 0.0, max_inner: int = 20000, max_outer: int = 12,
                       stall_factor: float = 0.5, max_fallback: int = 20000,
                       learned=None, projection: int = 0) -> dict:
        """One timestep solved to a relative FP64 true residual with one of
        the solver-replacement methods (cg64 | mixed | mixed-jacobi |
        mixed-learned | mixed-learned-coarse | mixed-learned-layers, the
        learned ones with `learned`, a learned.Net). projection > 0 starts
        from the A-norm best combination of u0 and up to that many solutions
        of this chunk's earlier solves (0: from u0, as the reference)."""
        x, y, hd, f = self.x, self.y, self.hd, self.f
        rx, ry = self.rx_ry()
        self.halos(["energy", "density"], 2)
        prm = TLSolveParams(METHODS[method], rel_tol, inner_tol, max_inner, max_outer,
                            stall_factor, max_fallback,
                            learned.h if learned is not None else None, projection)
        rep = TLSolveReport()
        self.call("tl_solve", x, y, hd, self.coefficient, rx, ry, C.byref(prm), f["p"], f["r"],
                  f["u"], f["u0"], f["w"], f["kx"], f["ky"], f["density"], f["energy"],
                  C.byref(rep))
        self.last_report = rep.as_dict()
        self.last_steps = rep.inner_steps + rep.fallback_steps
        self.solve_finished()
        return self.last_report

    def solve_finished(self) -> None:
        """TeaLeaf/drivers/solve_finished_driver.c:7-43."""
        x, y, hd, f = self.x, self.y, self.hd, self.f
        self.call("tl_calculate_residual", x, y, hd, f["u"], f["u0"], f["r"], f["kx"], f["ky"])
        norm = C.c_double(0.0)
        self.call("tl_calculate_2norm", x, y, hd, f["r"], C.byref(norm))
        self.residual_norm = norm.value
        self.call("tl_finalise", x, y, hd, f["u"], f["density"], f["energy"])
        self.halos(["p", "energy", "u"], 1)

    def summary(self) -> tuple[float, float, float, float]:
        out = [C.c_double(0.0) for _ in range(4)]
        self.call("tl_field_summary", self.x, self.y, self.hd, self.f["u"], self.f["density"],
                  self.f["energy0"], self.f["volume"], *[C.byref(o) for o in out])
        return tuple(o.value for o in out)

    def read(self, name: str) -> np.ndarray:
        n = {"x_area": (self.x + 1) * self.y, "y_area": self.x * (self.y + 1),
             "cell_x": self.x, "cell_y": self.y, "vertex_x": self.x + 1,
             "vertex_y": self.y + 1}.get(name, self.n)
        return self.ctx.download(self.f[name], n)

    def close(self) -> None:
        self.ctx.close()


def relative_residual(chunk: GpuChunk) -> float:
    """||u0 - A u||_2 / ||u0||_2 over the interior, in FP64 on the device."""
    f = chunk.f
    x, y, hd = chunk.x, chunk.y, chunk.hd
    chunk.call("tl_calculate_residual", x, y, hd, f["u"], f["u0"], f["r"], f["kx"], f["ky"])
    rr = C.c_double(0.0)
    bb = C.c_double(0.0)
    chunk.call("tl_calculate_2norm", x, y, hd, f["r"], C.byref(rr))
    chunk.call("tl_calculate_2norm", x, y, hd, f["u0"], C.byref(bb))
    return math.sqrt(rr.value / bb.value) if bb.value > 0 else math.sqrt(rr.value)


__all__ = ["GpuChunk", "parsed_states", "relative_residual", "check"]
