"""ctypes bindings of the CPU oracle (oracle/_build/libtl_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product. Function names mirror
the GPU C ABI (tl_* -> orc_*) with host numpy arrays in place of device
pointers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_build" / "libtl_oracle.so"
DRIVER = ORACLE_DIR / "_build" / "tealeaf_oracle"
REF_DRIVER = ORACLE_DIR / "_ref" / "tealeaf_ref"
# The reference sources: TEALEAF_REF, else a TeaLeaf tree beside this repository.
REFERENCE_SOURCES = Path(os.environ.get("TEALEAF_REF",
                                        ORACLE_DIR.parent.parent / "reference" / "TeaLeaf"))


class OrcState(C.Structure):
    _fields_ = [("density", C.c_double), ("energy", C.c_double), ("x_min", C.c_double),
                ("y_min", C.c_double), ("x_max", C.c_double), ("y_max", C.c_double),
                ("radius", C.c_double), ("geometry", C.c_int)]


_A = C.c_void_p   # host array (numpy .ctypes.data)
_D = C.c_double
_I = C.c_int
_PD = C.POINTER(C.c_double)

SIGNATURES = {
    "orc_reduce_sycl_order": ([_A, C.c_long], C.c_double),
    "orc_set_chunk_data_vertices": ([_I, _I, _I, _A, _A, _D, _D, _D, _D], None),
    "orc_set_chunk_data": ([_I, _I, _I, _A, _A, _A, _A, _A, _A, _A, _D, _D, _D, _D], None),
    "orc_set_chunk_initial_state": ([_I, _I, _D, _D, _A, _A], None),
    "orc_set_chunk_state": ([_I, _I, _I, C.POINTER(OrcState), _A, _A, _A, _A, _A, _A, _A], None),
    "orc_store_energy": ([_I, _I, _A, _A], None),
    "orc_update_face": ([_I, _I, _I, _A, _I, _I], None),
    "orc_pack_or_unpack": ([_I, _I, _I, _I, _I, _I, _A, _A], None),
    "orc_field_summary": ([_I, _I, _I, _A, _A, _A, _A, _PD, _PD, _PD, _PD], None),
    "orc_cg_init_u": ([_I, _I, _I, _A, _A, _A, _A, _A, _A], None),
    "orc_cg_init_k": ([_I, _I, _I, _A, _A, _A, _D, _D], None),
    "orc_cg_init_others": ([_I, _I, _I, _A, _A, _A, _A, _A, _A, _PD], None),
    "orc_cg_calc_w": ([_I, _I, _I, _A, _A, _A, _A, _PD], None),
    "orc_cg_calc_ur": ([_I, _I, _I, _A, _A, _A, _A, _D, _PD], None),
    "orc_cg_calc_p": ([_I, _I, _I, _D, _A, _A], None),
    "orc_cg_calc_w_fused": ([_I, _I, _I, _A, _A, _A, _A, _PD], None),
    "orc_cg_calc_ur_fused": ([_I, _I, _I, _A, _A, _A, _A, _D, _PD], None),
    "orc_cg_calc_p_fused": ([_I, _I, _I, _D, _A, _A], None),
    "orc_copy_u": ([_I, _I, _I, _A, _A], None),
    "orc_calculate_residual": ([_I, _I, _I, _A, _A, _A, _A, _A], None),
    "orc_calculate_2norm": ([_I, _I, _I, _A, _PD], None),
    "orc_finalise": ([_I, _I, _I, _A, _A, _A], None),
    "orc_jacobi_init": ([_I, _I, _I, _I, _D, _D, _A, _A, _A, _A, _A, _A], None),
    "orc_jacobi_copy_u": ([_I, _I, _A, _A], None),
    "orc_jacobi_iterate": ([_I, _I, _I, _A, _A, _A, _A, _A, _PD], None),
    "orc_cheby_init": ([_I, _I, _I, _D, _A, _A, _A, _A, _A, _A, _A], None),
    "orc_cheby_iterate": ([_I, _I, _I, _D, _D, _A, _A, _A, _A, _A, _A, _A], None),
    "orc_cheby_calc_u": ([_I, _I, _I, _A, _A], None),
    "orc_ppcg_init": ([_I, _I, _I, _D, _A, _A], None),
    "orc_ppcg_calc_ur": ([_I, _I, _I, _A, _A, _A, _A, _A], None),
    "orc_ppcg_calc_sd": ([_I, _I, _I, _D, _D, _D, _A, _A], None),
    "orc_num_threads": ([], _I),
    "orc_set_num_threads": ([_I], None),
}

_lib = None


def build(with_reference: bool | None = None) -> None:
    """Builds the oracle library and driver (and, where the reference sources
    exist, the reference driver linked with the oracle)."""
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "lib", "driver"], check=True,
                   capture_output=True)
    if with_reference is None:
        with_reference = REFERENCE_SOURCES.is_dir()
    if with_reference:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref",
                        f"TEALEAF_REF={REFERENCE_SOURCES}"], check=True, capture_output=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(with_reference=False)
        l = C.CDLL(str(LIB))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.argtypes = args
            fn.restype = res
        _lib = l
    return _lib


def a(arr: np.ndarray) -> int:
    assert arr.dtype == np.float64 and arr.flags.c_contiguous
    return arr.ctypes.data


def _pd(v: C.c_double):
    return C.byref(v)


class OracleChunk:
    """The CPU twin of exploringsycl_gb300.chunk.GpuChunk: the same sequence
    of kernel calls on host arrays, with the CG driver loop of
    TeaLeaf/drivers/cg_driver.c:7-124 written out in Python."""

    FIELDS = ["density0", "density", "energy0", "energy", "u", "u0", "p", "r", "mi", "w",
              "kx", "ky", "sd", "volume"]

    def __init__(self, deck):
        from exploringsycl_gb300.chunk import parsed_states  # states as parsed
        self.L = lib()
        self.deck = deck
        self.hd = deck.halo_depth or 2
        self.x = deck.x_cells + 2 * self.hd
        self.y = deck.y_cells + 2 * self.hd
        self.n = self.x * self.y
        self.dx = (deck.xmax - deck.xmin) / deck.x_cells
        self.dy = (deck.ymax - deck.ymin) / deck.y_cells
        self.coefficient = 1 if deck.coefficient in (None, "density") else 2
        self.f = {k: np.zeros(self.n) for k in self.FIELDS}
        self.f["x_area"] = np.zeros((self.x + 1) * self.y)
        self.f["y_area"] = np.zeros(self.x * (self.y + 1))
        self.f["cell_x"] = np.zeros(self.x)
        self.f["cell_y"] = np.zeros(self.y)
        self.f["vertex_x"] = np.zeros(self.x + 1)
        self.f["vertex_y"] = np.zeros(self.y + 1)
        self.states = parsed_states(deck)
        self.initialise()

    def p(self, name):
        return a(self.f[name])

    def halos(self, names, depth):
        for nm in names:
            for face in (0, 1, 3, 2):  # L, R, T, B
                self.L.orc_update_face(self.x, self.y, self.hd, self.p(nm), face, depth)

    def initialise(self):
        L, x, y, hd, d = self.L, self.x, self.y, self.hd, self.deck
        L.orc_set_chunk_data_vertices(x, y, hd, self.p("vertex_x"), self.p("vertex_y"), d.xmin,
                                      d.ymin, self.dx, self.dy)
        L.orc_set_chunk_data(x, y, hd, self.p("vertex_x"), self.p("vertex_y"), self.p("cell_x"),
                             self.p("cell_y"), self.p("volume"), self.p("x_area"),
                             self.p("y_area"), d.xmin, d.ymin, self.dx, self.dy)
        s0 = self.states[0]
        L.orc_set_chunk_initial_state(x, y, s0.energy, s0.density, self.p("energy0"),
                                      self.p("density"))
        for s in self.states[1:]:
            os_ = OrcState(s.density, s.energy, s.x_min, s.y_min, s.x_max, s.y_max, s.radius,
                           s.geometry)
            L.orc_set_chunk_state(x, y, hd, C.byref(os_), self.p("energy0"), self.p("density"),
                                  self.p("u"), self.p("cell_x"), self.p("cell_y"),
                                  self.p("vertex_x"), self.p("vertex_y"))
        self.halos(["density", "energy0", "energy"], 2)
        L.orc_store_energy(x, y, self.p("energy"), self.p("energy0"))

    def rx_ry(self):
        dt = self.deck.initial_timestep
        return dt / (self.dx * self.dx), dt / (self.dy * self.dy)

    def cg_timestep(self, max_iters=None, rel_tol=None, contract="exact"):
        """One timestep of the reference CG driver; returns the number of
        main steps executed and records pw/rrn of each. With rel_tol the stop
        rule becomes sqrt(rr) < rel_tol * ||u0||_2 instead of eps. contract
        'fused' uses the fused multiply-add kernels of the GPU's
        TL_FP64_FUSED persistent solve."""
        L, x, y, hd = self.L, self.x, self.y, self.hd
        fused = contract == "fused"
        calc_w = L.orc_cg_calc_w_fused if fused else L.orc_cg_calc_w
        calc_ur = L.orc_cg_calc_ur_fused if fused else L.orc_cg_calc_ur
        calc_p = L.orc_cg_calc_p_fused if fused else L.orc_cg_calc_p
        max_iters = self.deck.max_iters if max_iters is None else max_iters
        rx, ry = self.rx_ry()
        self.halos(["energy", "density"], 2)
        rro = C.c_double(0.0)
        L.orc_cg_init_u(x, y, self.coefficient, self.p("p"), self.p("r"), self.p("u"),
                        self.p("w"), self.p("density"), self.p("energy"))
        L.orc_cg_init_k(x, y, hd, self.p("w"), self.p("kx"), self.p("ky"), rx, ry)
        L.orc_cg_init_others(x, y, hd, self.p("kx"), self.p("ky"), self.p("p"), self.p("r"),
                             self.p("u"), self.p("w"), _pd(rro))
        self.rro0 = rro.value
        self.halos(["u", "p"], 1)
        L.orc_copy_u(x, y, hd, self.p("u"), self.p("u0"))
        eps = self.deck.eps
        if rel_tol is not None:
            bb = C.c_double(0.0)
            L.orc_calculate_2norm(x, y, hd, self.p("u0"), _pd(bb))
            eps = rel_tol * np.sqrt(bb.value)
        self.pw_hist, self.rrn_hist = [], []
        rro_v = rro.value
        steps = 0
        for tt in range(max_iters):
            pw = C.c_double(0.0)
            calc_w(x, y, hd, self.p("w"), self.p("p"), self.p("kx"), self.p("ky"), _pd(pw))
            alpha = rro_v / pw.value
            rrn = C.c_double(0.0)
            calc_ur(x, y, hd, self.p("u"), self.p("r"), self.p("p"), self.p("w"), alpha,
                    _pd(rrn))
            beta = rrn.value / rro_v
            calc_p(x, y, hd, beta, self.p("p"), self.p("r"))
            self.pw_hist.append(pw.value)
            self.rrn_hist.append(rrn.value)
            rro_v = rrn.value
            steps = tt + 1
            self.halos(["u", "p"], 1)
            if np.sqrt(abs(rrn.value)) < eps:
                break
        self.last_steps = steps
        self.solve_finished()
        return steps

    def solve_finished(self):
        L, x, y, hd = self.L, self.x, self.y, self.hd
        L.orc_calculate_residual(x, y, hd, self.p("u"), self.p("u0"), self.p("r"), self.p("kx"),
                                 self.p("ky"))
        nrm = C.c_double(0.0)
        L.orc_calculate_2norm(x, y, hd, self.p("r"), _pd(nrm))
        self.residual_norm = nrm.value
        L.orc_finalise(x, y, hd, self.p("u"), self.p("density"), self.p("energy"))
        self.halos(["p", "energy", "u"], 1)

    def summary(self):
        out = [C.c_double(0.0) for _ in range(4)]
        self.L.orc_field_summary(self.x, self.y, self.hd, self.p("u"), self.p("density"),
                                 self.p("energy0"), self.p("volume"), *[_pd(o) for o in out])
        return tuple(o.value for o in out)
