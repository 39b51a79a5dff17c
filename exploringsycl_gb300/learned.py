"""Learned preconditioner: data harvesting, training and the weights file.

All arithmetic runs in this project's CUDA kernels (include/tealeaf_gb300.h,
tl_net_*); Python only orchestrates.

* harvest(): seeded random-state problems (the deck distribution of
  deck.random_states) are initialised on the GPU; for each, plain FP64 CG is
  run for a few step counts and the residual after each is kept, packed to
  FP32, with the problem's FP32 coefficients kx, ky and s = D^-1/2. The
  problems' timestep sets the conduction regime: kx, ky are rx K with
  rx = dt / dx^2, so a 512^2 problem at dt = 0.004 (4096/512)^2 carries the
  couplings of a 4096^2 problem at the default dt = 0.004.
* uniform(): fields of one constant coupling c = rx K each, c log-uniform
  over the range of a random-state deck, for training on the operator away
  from material interfaces (the default: see train_cli).
* train(): Adam on random crops of those residuals, with the loss
  sum ||A M^-1 r - r||^2 / sum ||r||^2 over the batch, on the crop interiors.
  Residual crops may be replaced by white-noise probes, optionally smoothed
  by the operator's symbol (smooth_probes) so that the loss weighs the low
  frequencies, where CG converges slowly, more.
* Weights file: a .npz with the FP32 weight vector, the layout version and a
  SHA-256 of the weight bytes, checked on load.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import Context, check
from . import deck as dk

LAYOUT_VERSION = 1
N_LAYERS = 4
CH = 16
DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "precond_4x16.npz"
DEFAULT_RAW_WEIGHTS = DEFAULT_WEIGHTS.with_suffix(".f32")


def num_params() -> int:
    from . import load_library
    return int(load_library().tl_net_num_params())


def identity_weights(noise: float = 0.0, seed: int = 0) -> np.ndarray:
    """Weights for which C^T C = I, so that M^-1 = 2 D^-1 (Jacobi): layer 1
    puts 1/4 of the scaled residual on every channel, layers 2..4 are
    identities; plus optional noise. Layout: layer 1 [tap][co], layers 2..4
    [tap][ci][co]."""
    rng = np.random.default_rng(seed)
    w1 = np.zeros((9, CH), np.float32)
    w1[4, :] = 0.25
    ws = [w1.ravel()]
    for _ in range(3):
        w = np.zeros((9, CH, CH), np.float32)
        w[4] = np.eye(CH, dtype=np.float32)
        ws.append(w.ravel())
    out = np.concatenate(ws)
    if noise:
        out += (noise * rng.standard_normal(out.size)).astype(np.float32)
    return out


def save_weights(path: str | Path, w: np.ndarray, meta: dict | None = None) -> Path:
    w = np.ascontiguousarray(w, dtype=np.float32)
    digest = hashlib.sha256(w.tobytes()).hexdigest()
    p = Path(path)
    p.parent.mkdir(parents=True, exist_ok=True)
    np.savez(p, weights=w, version=np.int32(LAYOUT_VERSION), sha256=np.array(digest),
             meta=np.array(json.dumps(meta or {})))
    return p


def export_raw(w: np.ndarray, path: str | Path = DEFAULT_RAW_WEIGHTS) -> Path:
    """Writes the weights as the raw little-endian FP32 file that the run_*
    backend reads (deck key gb300_weights, or TL_WEIGHTS)."""
    p = Path(path)
    np.ascontiguousarray(w, dtype="<f4").tofile(p)
    return p


def load_weights(path: str | Path = DEFAULT_WEIGHTS) -> tuple[np.ndarray, dict]:
    """Loads and verifies a weights file (version and checksum)."""
    with np.load(Path(path), allow_pickle=False) as f:
        w = f["weights"].astype(np.float32)
        version = int(f["version"])
        digest = str(f["sha256"])
        meta = json.loads(str(f["meta"]))
    if version != LAYOUT_VERSION:
        raise ValueError(f"weights layout version {version}, expected {LAYOUT_VERSION}")
    if hashlib.sha256(w.tobytes()).hexdigest() != digest:
        raise ValueError("weights checksum mismatch (truncated or modified file)")
    if not np.all(np.isfinite(w)):
        raise ValueError("weights contain non-finite values")
    return w, meta


class Net:
    """The device network (tl_net)."""

    def __init__(self, ctx: Context, weights: np.ndarray | None = None):
        self.ctx = ctx
        self.lib = ctx.lib
        self.h = C.c_void_p()
        check(self.lib.tl_net_create(ctx.h, C.byref(self.h)), "tl_net_create")
        self.n = num_params()
        self.set(identity_weights() if weights is None else weights)

    def set(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.n
        check(self.lib.tl_net_set_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), self.n),
              "tl_net_set_weights")

    def get(self) -> np.ndarray:
        w = np.empty(self.n, np.float32)
        check(self.lib.tl_net_get_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), self.n),
              "tl_net_get_weights")
        return w

    def apply(self, H, W, B, r_dev, s_dev, z_dev) -> None:
        check(self.lib.tl_net_apply(self.h, H, W, B, r_dev, s_dev, z_dev), "tl_net_apply")

    def loss_grad(self, H, W, B, margin, r, s, kx, ky, want_grad=False):
        loss = C.c_double(0.0)
        g = np.empty(self.n, np.float32) if want_grad else None
        check(self.lib.tl_net_loss_grad(
            self.h, H, W, B, margin, r, s, kx, ky, C.byref(loss),
            g.ctypes.data_as(C.POINTER(C.c_float)) if want_grad else None), "tl_net_loss_grad")
        return loss.value, g

    def adam(self, lr: float) -> None:
        check(self.lib.tl_net_adam_step(self.h, lr), "tl_net_adam_step")

    def stencil(self) -> tuple[np.ndarray, float]:
        """The 17x17 stencil K of C^T C (rows dy = -8..8, columns dx = -8..8)
        and the FP16 scale of its tensor-core copy, both computed on the GPU."""
        k = np.empty(17 * 17, np.float32)
        ks = C.c_float(0.0)
        check(self.lib.tl_net_stencil(self.h, k.ctypes.data_as(C.POINTER(C.c_float)),
                                      C.byref(ks)), "tl_net_stencil")
        return k.reshape(17, 17), ks.value

    def apply_stencil(self, H, W, r_dev, s_dev, z_dev) -> None:
        """z = M^-1 r on one packed [H][W] field with the collapsed stencil."""
        check(self.lib.tl_net_apply_stencil(self.h, H, W, r_dev, s_dev, z_dev),
              "tl_net_apply_stencil")

    def pcg(self, H, W, kx_dev, ky_dev, b_dev, e_dev, work_dev, tol: float,
            max_iters: int) -> tuple[int, float]:
        """The learned PCG on packed [H][W] fields: A e = b to r.r <= tol^2 b.b
        or max_iters steps (work: 7 H*W floats). Returns (steps, final r.r)."""
        it = C.c_int(0)
        rr = C.c_double(0.0)
        check(self.lib.tl_net_pcg(self.h, H, W, kx_dev, ky_dev, b_dev, e_dev, work_dev, tol,
                                  max_iters, C.byref(it), C.byref(rr)), "tl_net_pcg")
        return it.value, rr.value

    def close(self) -> None:
        if self.h:
            self.lib.tl_net_destroy(self.h)
            self.h = C.c_void_p()


@dataclass
class Dataset:
    size: int                 # interior cells per side of each problem
    n_problems: int
    snapshots: tuple[int, ...]
    r: int                    # device FP32 [P*S][size][size]
    kx: int                   # device FP32 [P][size][size]
    ky: int
    s: int


def like_timestep(size: int, like: int) -> float:
    """The timestep that gives size^2 problems the rx = dt / dx^2 of like^2
    problems at the default timestep 0.004."""
    return 0.004 * (like / size) ** 2


def harvest(ctx: Context, n_problems: int, size: int = 512, snapshots=(16, 64, 200),
            seed0: int = 100000, timestep: float = 0.004) -> Dataset:
    """Residual snapshots of plain FP64 CG on seeded random-state problems."""
    from .chunk import GpuChunk
    n = size * size
    S = len(snapshots)
    ds = Dataset(size, n_problems, tuple(snapshots), ctx.alloc_f32(n * n_problems * S),
                 ctx.alloc_f32(n * n_problems), ctx.alloc_f32(n * n_problems),
                 ctx.alloc_f32(n * n_problems))
    chunk = None
    pw = np.zeros(max(snapshots))
    rr = np.zeros(max(snapshots))
    for prob in range(n_problems):
        d = dk.random_deck(size, seed=seed0 + prob, end_step=1, max_iters=max(snapshots),
                           initial_timestep=timestep)
        if chunk is None:
            chunk = GpuChunk(d, ctx=ctx)
        else:
            chunk.deck = d
            chunk.initialise()
        f, x, y, hd = chunk.f, chunk.x, chunk.y, chunk.hd
        rx, ry = chunk.rx_ry()
        for si, k in enumerate(snapshots):
            rro = C.c_double(0.0)
            steps = C.c_int(0)
            chunk.call("tl_cg_solve", x, y, hd, chunk.coefficient, rx, ry, 0.0, k, f["p"], f["r"],
                       f["u"], f["u0"], f["w"], f["kx"], f["ky"], f["density"], f["energy"],
                       C.byref(rro), pw.ctypes.data_as(C.POINTER(C.c_double)),
                       rr.ctypes.data_as(C.POINTER(C.c_double)), C.byref(steps))
            norm = C.c_double(0.0)
            chunk.call("tl_calculate_2norm", x, y, hd, f["r"], C.byref(norm))
            scale = 1.0 / max(np.sqrt(norm.value / n), 1e-300)
            dst = ds.r + 4 * n * (prob * S + si)
            check(ctx.lib.tl_pack_interior(ctx.h, x, y, hd, f["r"], scale, dst), "pack")
        off = 4 * n * prob
        check(ctx.lib.tl_pack_coefficients(ctx.h, x, y, hd, f["kx"], f["ky"], ds.kx + off,
                                           ds.ky + off, ds.s + off), "pack coefficients")
    ctx.synchronize()
    return ds


def coupling_range(like: int, density_range=(0.05, 200.0)) -> tuple[float, float]:
    """The couplings kx = rx (1/d_left + 1/d_right) / 2 of random-state decks
    (density coefficient) at like^2 cells and dt = 0.004."""
    rx = 0.004 / (10.0 / like) ** 2
    return rx / density_range[1], rx / density_range[0]


def uniform(ctx: Context, n_problems: int, size: int = 256,
            c_range: tuple[float, float] = coupling_range(4096), seed: int = 0) -> Dataset:
    """Constant-coefficient problems: problem p has the coupling c_p
    (log-uniform in c_range) on every face, s = (1 + 4 c_p)^-1/2, and white
    noise as its residual. Away from material interfaces the scaled operator
    S A S of every deck looks like one of these, and a translation-invariant
    stencil can only be fitted to that part of it: on harvested crops the
    cells within the stencil's reach of an interface dominate the loss and
    pull the fit away from what shortens the CG iteration."""
    rng = np.random.default_rng(seed)
    n = size * size
    c = np.exp(rng.uniform(np.log(c_range[0]), np.log(c_range[1]), n_problems))
    kx = np.repeat(c, n).astype(np.float32)
    s = np.repeat(1.0 / np.sqrt(1.0 + 4.0 * c), n).astype(np.float32)
    ds = Dataset(size, n_problems, (0,), ctx.alloc_f32(n * n_problems),
                 ctx.alloc_f32(n * n_problems), ctx.alloc_f32(n * n_problems),
                 ctx.alloc_f32(n * n_problems))
    ctx.upload_f32(ds.r, rng.standard_normal(n * n_problems).astype(np.float32))
    ctx.upload_f32(ds.kx, kx)
    ctx.upload_f32(ds.ky, kx)
    ctx.upload_f32(ds.s, s)
    return ds


def gather(ctx: Context, ds: Dataset, which: str, meta: np.ndarray, crop: int, out: int) -> None:
    """Crops of one dataset array into `out` ([B][crop][crop])."""
    src = {"r": ds.r, "kx": ds.kx, "ky": ds.ky, "s": ds.s}[which]
    m = np.ascontiguousarray(meta, dtype=np.int32)
    if which != "r":  # coefficient arrays are per problem, not per snapshot
        m = m.copy()
        m[:, 0] //= len(ds.snapshots)
    check(ctx.lib.tl_net_gather_crops(ctx.h, src, ds.size, ds.size,
                                      m.ctypes.data_as(C.POINTER(C.c_int)), m.shape[0], crop,
                                      crop, out), "gather")


def smooth_probes(noise: np.ndarray, c: np.ndarray, k: float) -> np.ndarray:
    """White-noise crops [B][H][W] filtered by a_c(theta)^(-k/2) and scaled
    to unit RMS, where a_c = (1 + 2c (2 - cos theta_x - cos theta_y)) /
    (1 + 4c) is the symbol of the scaled operator S A S for the constant
    coupling c[b] of crop b. Under the loss ||A M^-1 r - r||^2 such probes
    weigh the misfit at frequency theta by a_c^-k: the low frequencies, where
    CG converges slowly, count more than under white noise (k = 0). The
    filter is periodic over the crop; the loss leaves out a margin at the
    crop's edge."""
    B, H, W = noise.shape
    ty = 2.0 * np.pi * np.fft.fftfreq(H)[:, None]
    tx = 2.0 * np.pi * np.fft.fftfreq(W)[None, :]
    c = np.asarray(c, dtype=np.float64).reshape(B, 1, 1)
    a = (1.0 + 2.0 * c * (2.0 - np.cos(ty) - np.cos(tx))) / (1.0 + 4.0 * c)
    r = np.fft.ifft2(np.fft.fft2(noise.astype(np.float64)) * a ** (-0.5 * k)).real
    r /= np.sqrt(np.mean(r * r, axis=(1, 2), keepdims=True))
    return r.astype(np.float32)


def train(net: Net, ds: Dataset, steps: int = 2000, batch: int = 32, crop: int = 128,
          lr: float = 1e-3, margin: int = 9, seed: int = 0, log_every: int = 100,
          lr_decay_at: float = 0.7, noise_fraction: float = 0.0,
          probe_smoothing: float = 0.0) -> list[tuple[int, float]]:
    """Adam on random crops; returns (step, loss) samples. With
    noise_fraction > 0 that share of the residual crops is replaced by white
    noise on the same coefficient crops, so that the loss also weighs the
    upper part of the spectrum (a least-squares fit of M^-1 A to I over all
    modes) and not only the smooth modes that dominate CG residuals. With
    probe_smoothing = k > 0 that noise is filtered by smooth_probes with each
    crop's mean coupling, which weighs the misfit at low frequencies more."""
    ctx = net.ctx
    rng = np.random.default_rng(seed)
    n = batch * crop * crop
    bufs = {k: ctx.alloc_f32(n) for k in ("r", "kx", "ky", "s")}
    history = []
    n_samples = ds.n_problems * len(ds.snapshots)
    for it in range(steps):
        meta = np.stack([rng.integers(0, n_samples, batch),
                         rng.integers(0, ds.size - crop + 1, batch),
                         rng.integers(0, ds.size - crop + 1, batch)], axis=1)
        for k in bufs:
            gather(ctx, ds, k, meta, crop, bufs[k])
        n_noise = int(round(noise_fraction * batch))
        if n_noise:
            r_host = ctx.download_f32(bufs["r"], n).reshape(batch, crop, crop)
            noise = rng.standard_normal((n_noise, crop, crop)).astype(np.float32)
            if probe_smoothing > 0.0:
                kx = ctx.download_f32(bufs["kx"], n).reshape(batch, crop, crop)[:n_noise]
                noise = smooth_probes(noise, kx.mean(axis=(1, 2)), probe_smoothing)
            r_host[:n_noise] = noise
            ctx.upload_f32(bufs["r"], r_host)
        loss, _ = net.loss_grad(crop, crop, batch, margin, bufs["r"], bufs["s"], bufs["kx"],
                                bufs["ky"])
        step_lr = lr if it < lr_decay_at * steps else lr * 0.1
        net.adam(step_lr)
        if it % log_every == 0 or it == steps - 1:
            history.append((it, loss))
    return history


def evaluate_loss(net: Net, ds: Dataset, batch: int = 32, crop: int = 128, margin: int = 9,
                  seed: int = 12345, rounds: int = 4) -> float:
    ctx = net.ctx
    rng = np.random.default_rng(seed)
    n = batch * crop * crop
    bufs = {k: ctx.alloc_f32(n) for k in ("r", "kx", "ky", "s")}
    n_samples = ds.n_problems * len(ds.snapshots)
    tot = 0.0
    for _ in range(rounds):
        meta = np.stack([rng.integers(0, n_samples, batch),
                         rng.integers(0, ds.size - crop + 1, batch),
                         rng.integers(0, ds.size - crop + 1, batch)], axis=1)
        for k in bufs:
            gather(ctx, ds, k, meta, crop, bufs[k])
        loss, _ = net.loss_grad(crop, crop, batch, margin, bufs["r"], bufs["s"], bufs["kx"],
                                bufs["ky"])
        tot += loss
    return tot / rounds


def compare_methods(weights: np.ndarray, size: int, seeds, rel_tol: float = 1e-10,
                    timestep: float = 0.004,
                    methods=("mixed", "mixed-jacobi", "mixed-learned")) -> dict:
    """Inner steps (CG steps for cg64) and device time of the solves on
    fresh random-state problems of the given seeds, summed over the seeds."""
    from .chunk import GpuChunk
    out = {m: {"inner_steps": 0, "device_ms": 0.0, "fallbacks": 0} for m in methods}
    for seed in seeds:
        d = dk.random_deck(size, seed=seed, end_step=1, initial_timestep=timestep)
        for method in out:
            g = GpuChunk(d)
            net = Net(g.ctx, weights) if method.startswith("mixed-learned") else None
            try:
                rep = g.solve_timestep(method, rel_tol=rel_tol, learned=net)
                out[method]["inner_steps"] += rep["inner_steps"]
                out[method]["device_ms"] += rep["device_ms"]
                out[method]["fallbacks"] += rep["fallback_events"]
                out[method]["max_rel_residual"] = max(out[method].get("max_rel_residual", 0.0),
                                                      rep["final_rel_residual"])
            finally:
                if net:
                    net.close()
                g.close()
    return out


def train_cli(argv=None) -> None:
    """python -m exploringsycl_gb300.learned --out FILE [--problems N] ...

    Trains the network from Jacobi-equivalent weights on white-noise
    residuals and writes the weights file and its raw FP32 twin (.f32). The
    coefficient crops come from constant-coefficient fields with the
    couplings of like^2 random-state decks (--data uniform, the default;
    --like 4096 is the size the preconditioner runs at) or from N seeded
    512^2 random-state problems harvested in that regime (--data harvest).
    The evaluation solves fresh random-state problems either way."""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    ap.add_argument("--data", choices=["uniform", "harvest"], default="uniform")
    ap.add_argument("--problems", type=int, default=2000)
    ap.add_argument("--uniform-problems", type=int, default=64)
    ap.add_argument("--uniform-size", type=int, default=256)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--like", type=int, default=4096,
                    help="harvest with the timestep that gives the problems the rx = dt/dx^2 "
                         "of like^2 problems at dt = 0.004")
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed0", type=int, default=100000)
    ap.add_argument("--snapshots", default="2,8,32",
                    help="CG step counts at which residuals are harvested")
    ap.add_argument("--noise-fraction", type=float, default=1.0)
    ap.add_argument("--probe-smoothing", type=float, default=1.0,
                    help="k: filter the noise probes by a^(-k/2) (0: white noise; the "
                         "committed weights use k = 1)")
    ap.add_argument("--eval-size", type=int, default=1024)
    ap.add_argument("--eval-size-small", type=int, default=512)
    ap.add_argument("--eval-seeds", default="7,8")
    args = ap.parse_args(argv)
    ctx = Context(0)
    t0 = time.time()
    dt = like_timestep(args.size, args.like)
    c_range = coupling_range(args.like)
    if args.data == "uniform":
        ds = uniform(ctx, args.uniform_problems, size=args.uniform_size, c_range=c_range,
                     seed=args.seed0)
    else:
        ds = harvest(ctx, args.problems, size=args.size, seed0=args.seed0,
                     snapshots=tuple(int(v) for v in args.snapshots.split(",")), timestep=dt)
    t1 = time.time()
    net = Net(ctx, identity_weights(noise=1e-3, seed=7))
    before = evaluate_loss(net, ds, crop=args.crop)
    hist = train(net, ds, steps=args.steps, batch=args.batch, crop=args.crop, lr=args.lr,
                 noise_fraction=args.noise_fraction, probe_smoothing=args.probe_smoothing)
    after = evaluate_loss(net, ds, crop=args.crop)
    t2 = time.time()
    meta = {"data": args.data, "like": args.like, "coupling_range": list(c_range),
            "problems": ds.n_problems, "size": ds.size, "timestep": dt,
            "snapshots": list(ds.snapshots),
            "steps": args.steps, "batch": args.batch, "crop": args.crop, "lr": args.lr,
            "seed0": args.seed0, "noise_fraction": args.noise_fraction,
            "probe_smoothing": args.probe_smoothing, "loss_jacobi": before, "loss_trained": after,
            "harvest_s": t1 - t0, "train_s": t2 - t1, "history": hist[::max(1, len(hist) // 20)]}
    w = net.get()
    seeds = [int(v) for v in args.eval_seeds.split(",")]
    meta["eval"] = {"size": args.eval_size, "seeds": seeds,
                    "results": compare_methods(w, args.eval_size, seeds)}
    meta["eval_small"] = {"size": args.eval_size_small, "seeds": seeds,
                          "results": compare_methods(w, args.eval_size_small, seeds)}
    dt_small = like_timestep(args.eval_size_small, args.like)
    meta["eval_like"] = {"size": args.eval_size_small, "timestep": dt_small, "seeds": seeds,
                         "results": compare_methods(w, args.eval_size_small, seeds,
                                                    timestep=dt_small)}
    save_weights(args.out, w, meta)
    export_raw(w, Path(args.out).with_suffix(".f32"))
    print(json.dumps({k: v for k, v in meta.items() if k != "history"}))
    net.close()
    ctx.close()


def evaluate_cli(argv=None) -> None:
    """python -m exploringsycl_gb300.learned evaluate [--sizes 1024,4096] ...

    Solves one timestep of fresh random-state problems (seeds the network
    was neither trained nor tuned on) to the relative FP64 true residual
    1e-10 with plain FP64 CG (cg64), the FP32-inner CG and Jacobi-PCG in FP64
    refinement, and the learned PCG (without and with the coarse level) in
    FP64 refinement, each from u0; prints, per size and
    per seed, each method's steps, device time, fall-backs and final
    residual as one JSON line."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--weights", default=str(DEFAULT_WEIGHTS))
    ap.add_argument("--sizes", default="1024,4096")
    ap.add_argument("--seeds", default="31,32,33")
    ap.add_argument("--seeds-large", default="31",
                    help="seeds for sizes above 2048 (each plain FP64 CG solve takes seconds)")
    args = ap.parse_args(argv)
    w, meta = load_weights(args.weights)
    methods = ("cg64", "mixed", "mixed-jacobi", "mixed-learned", "mixed-learned-coarse")
    result = {"weights": Path(args.weights).name, "rel_tol": 1e-10, "timestep": 0.004,
              "training": {k: meta.get(k) for k in ("data", "like", "seed0", "steps",
                                                    "probe_smoothing")},
              "sizes": {}}
    for size in (int(v) for v in args.sizes.split(",")):
        seeds = [int(v) for v in (args.seeds_large if size > 2048 else args.seeds).split(",")]
        per_seed = {seed: compare_methods(w, size, [seed], methods=methods) for seed in seeds}
        result["sizes"][size] = {"seeds": seeds, "per_seed": per_seed}
    print(json.dumps(result))


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "evaluate":
        evaluate_cli(sys.argv[2:])
    else:
        train_cli()
