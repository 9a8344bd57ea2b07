"""The learned PCG preconditioner: Newton-system capture, training and weights.

The network (csrc/gpu/learned.cuh) emits the factor G of
P = G^T G + eps D^{-1} on the Newton system's own sparsity. Its forward and
backward passes are the library's own kernels, reached through
ppf_learned_loss_grad; PyTorch only holds the device buffers and runs Adam on
the fp32 master copy of the weights, whose bf16 rounding is what the kernels
read. Training data are the Newton systems the solver itself assembles
(ppf_debug_newton_system), and the loss is Kaporin's condition number of
Ĝ Â Ĝ^T, estimated with random +-1 probes.

The reference has no learned preconditioner: its PCG uses block-Jacobi
(crates/ppf-cts-solver/src/cpp/solver/solver.cu:357-400), which stays the
fallback of every learned solve.

Usage (on a GPU):
    python -m ppf_gb300.learned train --out weights.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time
from pathlib import Path

import numpy as np

from . import abi, scenes
from ._lib import f32p, f32p_opt, product, u32p, u32p_opt
from .session import Session, SolverError

N_WEIGHTS = 12592
OFF_W0, OFF_W1, OFF_WH, OFF_WF, OFF_WO = 0, 512, 8192, 12032, 12544
WEIGHTS_FILE = Path(__file__).resolve().parent / "weights" / "learned_precond.npz"

_declared = set()


def _declare(lib):
    if id(lib) in _declared:
        return
    P = C.c_void_p
    lib.ppf_set_learned_weights.restype = C.c_int
    lib.ppf_set_learned_weights.argtypes = [np.ctypeslib.ndpointer(np.uint16, flags="C"), C.c_uint]
    lib.ppf_learned_add_sample.restype = C.c_int
    lib.ppf_learned_add_sample.argtypes = [C.c_uint, u32p, u32p, f32p, u32p_opt, u32p_opt,
                                           f32p_opt, u32p, f32p]
    lib.ppf_learned_clear_samples.restype = None
    lib.ppf_learned_clear_samples.argtypes = []
    lib.ppf_learned_sample_info.restype = C.c_int
    lib.ppf_learned_sample_info.argtypes = [C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                            C.POINTER(C.c_uint)]
    lib.ppf_learned_forward.restype = C.c_int
    lib.ppf_learned_forward.argtypes = [C.c_int, P, f32p_opt, f32p_opt]
    lib.ppf_learned_loss_grad.restype = C.c_int
    lib.ppf_learned_loss_grad.argtypes = [C.c_int, P, P, C.c_uint, P, C.POINTER(C.c_float), P]
    lib.ppf_learned_tensor_path.restype = C.c_int
    lib.ppf_learned_tensor_path.argtypes = [C.c_int]
    lib.ppf_learned_tc_status.restype = C.c_uint
    lib.ppf_learned_tc_status.argtypes = []
    lib.ppf_debug_vertex_info.restype = None
    lib.ppf_debug_vertex_info.argtypes = [f32p_opt, u32p_opt]
    lib.ppf_debug_factor_diag.restype = None
    lib.ppf_debug_factor_diag.argtypes = [f32p]
    lib.ppf_debug_system.restype = None
    lib.ppf_debug_system.argtypes = [u32p_opt, u32p_opt, f32p_opt, u32p_opt, u32p_opt, f32p_opt,
                                     f32p_opt, f32p_opt, u32p_opt, u32p_opt, u32p_opt, u32p_opt]
    lib.ppf_debug_system_sizes.argtypes = [u32p]
    _declared.add(id(lib))


def lib():
    L = product()
    _declare(L)
    return L


# ---- weights ----------------------------------------------------------------------------


def init_weights(seed: int = 0) -> np.ndarray:
    """Initial fp32 weights: uniform +-1/sqrt(fan in) per layer over the used
    inputs, a head scaled by 0.1, and the edge output biased so that alpha
    starts at 1/2 (the first-order factor) and d at 1."""
    rng = np.random.default_rng(seed)
    w = np.zeros(N_WEIGHTS, np.float32)

    def fill(off, rows, cols, used_rows, used_cols, scale=1.0):
        m = w[off:off + rows * cols].reshape(rows, cols)
        m[:used_rows, :used_cols] = scale * rng.uniform(-1, 1, (used_rows, used_cols)) / np.sqrt(used_cols)

    fill(OFF_W0, 32, 16, 32, 16)
    for l in range(3):
        fill(OFF_W1 + l * 32 * 80, 32, 80, 32, 65)
    fill(OFF_WH, 80, 48, 65, 33, 0.1)
    fill(OFF_WF, 32, 16, 32, 11)
    w[OFF_WO:OFF_WO + 32] = 0.1 * rng.uniform(-1, 1, 32) / np.sqrt(32)
    w[OFF_WO + 32] = np.log(1.0 / 3.0)  # 2 sigmoid(ln 1/3) = 1/2
    return w


def to_bf16_bits(w) -> np.ndarray:
    """fp32 -> bf16 bit patterns, rounding to nearest even."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def load_weights(path=None) -> np.ndarray:
    """fp32 master weights of a trained network (the packaged ones by default)."""
    with np.load(Path(path) if path else WEIGHTS_FILE) as z:
        w = np.asarray(z["w"], np.float32)
    if w.size != N_WEIGHTS:
        raise ValueError(f"weights have {w.size} values, the network needs {N_WEIGHTS}")
    return w


def use_weights(w=None) -> None:
    """Loads weights into the solver (the packaged trained ones by default), so
    Session.set_preconditioner(abi.PRECOND_LEARNED) becomes available."""
    bits = to_bf16_bits(load_weights() if w is None else w)
    if lib().ppf_set_learned_weights(bits, bits.size) != 0:
        raise ValueError("the library rejected the weights")


# ---- Newton systems as samples -------------------------------------------------------------


def capture_system(n: int) -> dict:
    """The Newton system of the current state of the live session, assembled
    by the solver itself: its fixed pattern, contact blocks, right-hand side,
    masses, Dirichlet mask, and the block-Jacobi iteration count."""
    L = lib()
    dx = np.empty(3 * n, np.float32)
    it, rr = C.c_uint(), C.c_float()
    L.ppf_debug_newton_system(dx, C.byref(it), C.byref(rr))
    sizes = np.zeros(6, np.uint32)
    L.ppf_debug_system_sizes(sizes)
    nf, nd = int(sizes[0]), int(sizes[1])
    s = {
        "f_off": np.zeros(n + 1, np.uint32), "f_col": np.zeros(max(nf, 1), np.uint32),
        "f_val": np.zeros(9 * max(nf, 1), np.float32),
        "d_off": np.zeros(n + 1, np.uint32), "d_col": np.zeros(max(nd, 1), np.uint32),
        "d_val": np.zeros(9 * max(nd, 1), np.float32), "force": np.zeros(3 * n, np.float32),
    }
    L.ppf_debug_system(s["f_off"], s["f_col"], s["f_val"], s["d_off"], s["d_col"], s["d_val"],
                       None, s["force"], None, None, None, None)
    s["f_col"], s["f_val"] = s["f_col"][:nf], s["f_val"][:9 * nf]
    s["d_col"], s["d_val"] = s["d_col"][:nd], s["d_val"][:9 * nd]
    s["mass"] = np.zeros(n, np.float32)
    s["dof"] = np.zeros(n, np.uint32)
    L.ppf_debug_vertex_info(s["mass"], s["dof"])
    s["n"] = n
    s["bj_iters"] = int(it.value)
    return s


def collect(scene, steps: int, every: int = 3, start: int = 1, pin_motion=None):
    """Steps a scene with block-Jacobi and yields the Newton system captured at
    the start of every `every`-th step from `start` on."""
    sess = Session(scene, pin_motion=pin_motion)
    sess.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
    n = scene.vertex_count
    for k in range(steps):
        if k >= start and (k - start) % every == 0:
            yield capture_system(n)
        try:
            r = sess.step()
        except SolverError:
            break
        if not r.success():
            break


def add_sample(s: dict) -> int:
    d_off = s["d_off"] if s["d_off"][-1] else None
    idx = lib().ppf_learned_add_sample(
        int(s["n"]), s["f_off"], s["f_col"], s["f_val"], d_off,
        s["d_col"] if d_off is not None else None, s["d_val"] if d_off is not None else None,
        s["dof"], s["mass"])
    if idx < 0:
        raise ValueError("the library rejected the sample")
    return idx


# ---- training -------------------------------------------------------------------------------


class Trainer:
    """Adam on the fp32 master weights; loss and gradient from the library's
    kernels on the samples kept on the device."""

    def __init__(self, ids, sizes, seed: int = 0, lr: float = 3e-3, probes: int = 8, w0=None):
        import torch

        self.torch = torch
        self.dev = torch.device("cuda")
        self.ids = list(ids)
        self.n = [int(x) for x in sizes]
        self.param = torch.nn.Parameter(torch.tensor(
            init_weights(seed) if w0 is None else np.asarray(w0, np.float32), device=self.dev))
        self.opt = torch.optim.Adam([self.param], lr=lr)
        self.probes = probes
        self.gen = torch.Generator(device=self.dev)
        self.gen.manual_seed(seed)

    def loss_grad(self, k: int, w_bf16=None):
        """(loss, fp32 gradient tensor) of sample k at the current weights."""
        torch = self.torch
        wb = (self.param.detach().to(torch.bfloat16) if w_bf16 is None else w_bf16).contiguous()
        pr = torch.randint(0, 2, (self.probes, self.n[k], 3), generator=self.gen,
                           device=self.dev, dtype=torch.int32).to(torch.float32) * 2 - 1
        grad = torch.empty(N_WEIGHTS, dtype=torch.float32, device=self.dev)
        loss = C.c_float()
        rc = lib().ppf_learned_loss_grad(self.ids[k], wb.data_ptr(), pr.data_ptr(), self.probes,
                                         grad.data_ptr(), C.byref(loss),
                                         torch.cuda.current_stream().cuda_stream)
        if rc != 0:
            raise RuntimeError("ppf_learned_loss_grad failed")
        return float(loss.value), grad

    def step(self, k: int, lr: float = None) -> float:
        loss, grad = self.loss_grad(k)
        if lr is not None:
            for group in self.opt.param_groups:
                group["lr"] = lr
        self.opt.zero_grad()
        self.param.grad = grad
        self.opt.step()
        return loss

    def weights(self) -> np.ndarray:
        return self.param.detach().cpu().numpy().astype(np.float32)


def sample_loss(ids, w, probes: int = 16, seed: int = 1) -> list:
    """Mean Kaporin loss of weights w on already added samples."""
    import torch

    dev = torch.device("cuda")
    wb = torch.tensor(w, device=dev).to(torch.bfloat16).contiguous()
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    out = []
    grad = torch.empty(N_WEIGHTS, dtype=torch.float32, device=dev)
    for k in ids:
        n = C.c_uint()
        lib().ppf_learned_sample_info(k, C.byref(n), None, None)
        pr = torch.randint(0, 2, (probes, n.value, 3), generator=gen, device=dev,
                           dtype=torch.int32).to(torch.float32) * 2 - 1
        loss = C.c_float()
        lib().ppf_learned_loss_grad(k, wb.data_ptr(), pr.data_ptr(), probes, grad.data_ptr(),
                                    C.byref(loss), torch.cuda.current_stream().cuda_stream)
        out.append(float(loss.value))
    return out


def training_scenes(preset: str = "small"):
    """The scenes the training systems come from, as (name, factory, steps,
    every); factory() returns (scene, pin_motion).

    small: stacked cloth sheets (8 sheets of 128 x 128 over a cube) at seeds
    1-3, a 128 x 256 twisted tube, and 256^2 cloth over 12 spheres at seeds
    1-2 (145 systems).
    full: the 131,072-vertex stacked sheets at seeds 1-26 (seeded rotations
    and offsets), every second step of 90, 256 x 512 twisted tubes whose end
    rings turn at a seeded rate in [1.5, 2.5] rad/s (seeds 1-16, the first 45
    steps), and the two sphere fields: about 2,000 systems."""
    if preset == "small":
        out = [(f"stacked_sheets_128x8_seed{k}",
                (lambda k=k: scenes.stacked_sheets(side=128, sheets=8, seed=k)), 90, 3)
               for k in (1, 2, 3)]
        out.append(("twisted_tube_128x256", lambda: scenes.twisted_tube(around=128, along=256),
                    45, 3))
    else:
        out = [(f"stacked_sheets_128x8_seed{k}",
                (lambda k=k: scenes.stacked_sheets(side=128, sheets=8, seed=k)), 90, 2)
               for k in range(1, 27)]
        rng = np.random.default_rng(2024)
        for k in range(1, 17):
            omega = float(rng.uniform(1.5, 2.5))
            out.append((f"twisted_tube_256x512_seed{k}",
                        (lambda om=omega: scenes.twisted_tube(around=256, along=512, omega=om)),
                        45, 1))
    out += [(f"sphere_field_256_seed{k}",
             (lambda k=k: scenes.sphere_field(side=256, spheres=12, seed=k)), 60, 3)
            for k in (1, 2)]
    return out


def held_out_scenes():
    """Scenes of none of the training seeds, for comparing preconditioners."""
    return {
        "stacked_sheets_64x8_seed11": lambda: scenes.stacked_sheets(side=64, sheets=8, seed=11),
        "sphere_field_256_seed7": lambda: scenes.sphere_field(side=256, spheres=12, seed=7),
    }


def compare(scene_fn, steps: int, weights=None) -> dict:
    """PCG iterations, solves, block-Jacobi fallbacks and PCG ms of the same
    steps solved with block-Jacobi, the first-order factor and the learned
    factor (weights: fp32 master weights, the packaged ones by default)."""
    use_weights(weights)
    out = {}
    for name, kind in (("block_jacobi", abi.PRECOND_BLOCK_JACOBI),
                       ("first_order", abi.PRECOND_FIRST_ORDER),
                       ("learned", abi.PRECOND_LEARNED),
                       ("fsai", abi.PRECOND_FSAI)):
        sc, motion = scene_fn()
        sess = Session(sc, pin_motion=motion)
        sess.set_preconditioner(kind)
        it = solves = fb = 0
        ms = 0.0
        for _ in range(steps):
            if not sess.step(fetch=False).success():
                break
            st = sess.stats()
            it += st.pcg_iters_total
            solves += st.pcg_solves
            fb += st.fallbacks
            ms += st.pcg_ms_total
        sess.set_preconditioner(abi.PRECOND_BLOCK_JACOBI)
        out[name] = {"pcg_iters": it, "solves": solves, "fallbacks": fb,
                     "pcg_ms": round(ms, 2)}
        del sess, sc
    return out


def train_main(argv=None):
    ap = argparse.ArgumentParser(description="train the learned PCG preconditioner on a GPU")
    ap.add_argument("--out", required=True)
    ap.add_argument("--iters", type=int, default=6000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4,
                    help="cosine decay of the learning rate down to this value")
    ap.add_argument("--probes", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--preset", choices=["small", "full"], default="small")
    ap.add_argument("--systems", type=int, default=2000, help="stop collecting at this many")
    ap.add_argument("--min-free-gb", type=float, default=24.0,
                    help="stop collecting when less device memory than this is free")
    a = ap.parse_args(argv)
    import torch

    t0 = time.time()
    lib().ppf_learned_clear_samples()
    ids, sizes, names = [], [], []
    for name, factory, steps, every in training_scenes(a.preset):
        if len(ids) >= a.systems or torch.cuda.mem_get_info()[0] < a.min_free_gb * 2**30:
            break
        sc, motion = factory()
        k0 = len(ids)
        for s in collect(sc, steps, every=every, pin_motion=motion):
            ids.append(add_sample(s))
            sizes.append(int(s["n"]))
            names.append(name)
            if len(ids) >= a.systems or torch.cuda.mem_get_info()[0] < a.min_free_gb * 2**30:
                break
        print(f"{name}: {len(ids) - k0} systems ({time.time() - t0:.0f} s, "
              f"{torch.cuda.mem_get_info()[0] / 2**30:.0f} GB free)", flush=True)
        del sc
    rng = np.random.default_rng(a.seed)
    held = set(rng.choice(len(ids), size=max(1, len(ids) // 10), replace=False).tolist())
    train = [i for i in range(len(ids)) if i not in held]
    test_ids = [ids[i] for i in sorted(held)]
    tr = Trainer([ids[i] for i in train], [sizes[i] for i in train], seed=a.seed, lr=a.lr,
                 probes=a.probes)
    before = float(np.mean(sample_loss(test_ids, tr.weights())))
    losses = []
    for it in range(a.iters):
        lr = a.lr_final + 0.5 * (a.lr - a.lr_final) * (1 + np.cos(np.pi * it / max(1, a.iters)))
        losses.append(tr.step(int(rng.integers(len(train))), lr=lr))
        if it % 200 == 0:
            print(f"iter {it}: loss {np.mean(losses[-200:]):.4f} ({time.time() - t0:.0f} s)",
                  flush=True)
    after = float(np.mean(sample_loss(test_ids, tr.weights())))
    meta = {"systems": len(ids), "train": len(train), "held_out": len(test_ids),
            "iters": a.iters, "lr": a.lr, "lr_final": a.lr_final, "probes": a.probes,
            "preset": a.preset, "held_out_loss_init": before, "held_out_loss_trained": after,
            "scenes": sorted(set(names)), "seconds": time.time() - t0}
    print(json.dumps(meta), flush=True)
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    np.savez(a.out, w=tr.weights(), meta=json.dumps(meta))
    lib().ppf_learned_clear_samples()


def bench_main(argv=None):
    """Times the network on one Newton system of a stacked-sheets scene: the
    inference pass (features, layers, edge head on every upper entry) and one
    training step (forward, Kaporin loss, backward), with CUDA events; prints
    one JSON line."""
    import torch

    ap = argparse.ArgumentParser(description="time the learned preconditioner's kernels")
    ap.add_argument("--side", type=int, default=128)
    ap.add_argument("--sheets", type=int, default=8)
    ap.add_argument("--steps", type=int, default=15, help="time steps before the capture")
    ap.add_argument("--iters", type=int, default=50)
    ap.add_argument("--probes", type=int, default=8)
    ap.add_argument("--tensor-path", choices=["tc", "sync"], default=None,
                    help="forward layers as tcgen05 or mma.sync tiles (default: the library's)")
    a = ap.parse_args(argv)
    if a.tensor_path:
        lib().ppf_learned_tensor_path(1 if a.tensor_path == "tc" else 0)
    sc, _ = scenes.stacked_sheets(side=a.side, sheets=a.sheets, seed=1)
    s = next(iter(collect(sc, a.steps + 1, every=a.steps + 1, start=a.steps)))
    L = lib()
    L.ppf_learned_clear_samples()
    k = add_sample(s)
    n, E = C.c_uint(), C.c_uint()
    L.ppf_learned_sample_info(k, C.byref(n), C.byref(E), None)
    w = load_weights() if WEIGHTS_FILE.exists() else init_weights(0)
    tr = Trainer([k], [n.value], probes=a.probes, w0=w)
    wb = torch.tensor(w, device="cuda").to(torch.bfloat16).contiguous()
    alpha = np.zeros(E.value, np.float32)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.iters):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / a.iters

    fwd_ms = timed(lambda: L.ppf_learned_forward(k, wb.data_ptr(), None, None))
    step_ms = timed(lambda: tr.loss_grad(0, wb))
    L.ppf_learned_forward(k, wb.data_ptr(), alpha, None)
    nn = n.value
    # dense-layer flops per forward pass: 2 x rows x in x out
    flops = 2 * nn * (16 * 32 + 3 * 80 * 32 + 48 * 80)
    out = {"workload": f"stacked sheets {a.sheets} x {a.side}^2, Newton system after {a.steps} steps",
           "vertices": nn, "upper_entries": E.value,
           "live_edges": int((alpha != 0).sum()),
           "contact_blocks": int(s["d_off"][-1]),
           "inference_ms": round(fwd_ms, 4), "train_step_ms": round(step_ms, 4),
           "probes": a.probes, "dense_layer_gflop_per_forward": round(flops / 1e9, 3),
           "tensor_path": "tcgen05" if L.ppf_learned_tensor_path(-1) else "mma.sync",
           "tc_status": int(L.ppf_learned_tc_status()),
           "note": "inference_ms: features, the four layers and the edge head on every "
                   "upper entry, one device synchronization per call; the solver runs the "
                   "same kernels when it builds the learned factor"}
    print(json.dumps(out), flush=True)
    L.ppf_learned_clear_samples()


if __name__ == "__main__":
    import sys

    def eval_main(argv):
        ap = argparse.ArgumentParser(description="compare preconditioners on held-out scenes")
        ap.add_argument("--weights", default=None)
        ap.add_argument("--steps", type=int, default=30)
        a = ap.parse_args(argv)
        w = load_weights(a.weights)
        for name, fn in held_out_scenes().items():
            print(json.dumps({"scene": name, "steps": a.steps, **compare(fn, a.steps, w)}),
                  flush=True)

    cmds = {"train": train_main, "bench": bench_main, "eval": eval_main}
    if len(sys.argv) < 2 or sys.argv[1] not in cmds:
        raise SystemExit("usage: python -m ppf_gb300.learned train --out FILE [--iters N]\n"
                         "       python -m ppf_gb300.learned bench [--side N] [--iters N]\n"
                         "       python -m ppf_gb300.learned eval [--weights FILE]")
    cmds[sys.argv[1]](sys.argv[2:])
