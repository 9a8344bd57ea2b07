"""The learned PCG preconditioner (csrc/gpu/learned.cu).

CPU: the oracle's hand-derived gradient of the Kaporin loss against finite
differences (in exact arithmetic), and its loss against a dense evaluation.
GPU: the kernels' forward pass and gradient against the oracle on the same
system and probes; the learned factor used by the solver; training on the
GPU lowering the loss; what the packaged trained network gains over the
methods without it on a held-out scene; trajectory invariants.
"""
import ctypes as C

import numpy as np
import pytest

import learned_cases
from oracle import learned as OL


def _weights(seed=0):
    from ppf_gb300 import learned as PL

    return PL.init_weights(seed)


# ---- CPU: the oracle itself -------------------------------------------------------------------


def test_oracle_loss_matches_dense_kaporin_estimate():
    s = learned_cases.synthetic()
    g = learned_cases.graph(s)
    w = _weights(1)
    f = OL.forward(g, w)
    pr = learned_cases.probes(g.n, W=6)
    L, T, _, _ = OL.loss(g, f["alpha"], f["d"], pr)
    G = OL.factor_dense(g, f["alpha"].astype(np.float64), f["d"].astype(np.float64))
    # dense Â on the free dofs
    n = g.n
    A = np.zeros((3 * n, 3 * n))
    aii = OL._mul(OL._mul(g.cinv, g.A_ii), g.cinv.transpose(0, 2, 1))
    for i in range(n):
        if g.free[i]:
            A[3 * i:3 * i + 3, 3 * i:3 * i + 3] = aii[i]
    for e in np.nonzero(g.live)[0]:
        hi, lo = g.hi[e], g.lo[e]
        A[3 * hi:3 * hi + 3, 3 * lo:3 * lo + 3] = g.ah[e]
        A[3 * lo:3 * lo + 3, 3 * hi:3 * hi + 3] = g.ah[e].T
    M = G @ A @ G.T
    wv = (pr.astype(np.float64) * g.free[None, :, None]).reshape(pr.shape[0], -1)
    T_dense = np.mean([x @ M @ x for x in wv])
    assert abs(T - T_dense) <= 1e-5 * abs(T_dense)
    N = 3 * g.n_free
    L_dense = np.log(T_dense / N) - 2.0 / g.n_free * np.log(f["d"][g.free].astype(np.float64)).sum()
    assert abs(L - L_dense) < 1e-6


def test_oracle_gradient_matches_finite_differences():
    s = learned_cases.synthetic(seed=2)
    g = learned_cases.graph(s)
    w = _weights(3).astype(np.float32)
    pr = learned_cases.probes(g.n, W=4, seed=5)
    rng = np.random.default_rng(7)
    with OL.exact_arithmetic():
        L0, grad, _ = OL.loss_and_grad(g, w, pr)
        used = np.nonzero(grad != 0)[0]
        assert used.size > 1000
        errs = []
        for _ in range(6):
            d = np.zeros_like(w)
            d[used] = rng.normal(0, 1, used.size)
            d /= np.linalg.norm(d)
            eps = 2e-3
            lp = OL.loss_and_grad(g, (w + eps * d).astype(np.float32), pr)[0]
            lm = OL.loss_and_grad(g, (w - eps * d).astype(np.float32), pr)[0]
            fd = (lp - lm) / (2 * eps)
            an = float(grad.astype(np.float64) @ d)
            errs.append(abs(fd - an) / max(abs(an), 1e-3))
    assert np.median(errs) < 2e-2, errs


# ---- GPU ----------------------------------------------------------------------------------------


def _add(lib, s):
    from ppf_gb300 import learned as PL

    return PL.add_sample(s)


@pytest.fixture(scope="module")
def torch_cuda(product_lib):
    torch = pytest.importorskip("torch")
    return torch


@pytest.mark.gpu
def test_gpu_forward_matches_oracle(product_lib, torch_cuda):
    from ppf_gb300 import learned as PL

    torch = torch_cuda
    PL.lib().ppf_learned_clear_samples()
    s = learned_cases.synthetic(n=300, seed=4)
    g = learned_cases.graph(s)
    k = _add(product_lib, s)
    w = _weights(2)
    wb = torch.tensor(w, device="cuda").to(torch.bfloat16).contiguous()
    E = len(g.lo)
    alpha = np.zeros(E, np.float32)
    q = np.zeros(g.n, np.float32)
    assert PL.lib().ppf_learned_forward(k, wb.data_ptr(), alpha, q) == 0
    f = OL.forward(g, w)
    qo = f["q"]
    assert np.abs(q - qo)[g.free].max() <= 2e-2 * max(1.0, np.abs(qo).max()), np.abs(q - qo).max()
    assert np.abs(alpha - f["alpha"]).max() < 2e-2
    assert np.abs(alpha - f["alpha"]).mean() < 2e-3
    assert np.all(alpha[~g.live] == 0)


@pytest.mark.gpu
def test_tcgen05_layers_match_mma_sync(product_lib, torch_cuda):
    """The forward layers as tcgen05 tiles (tensor memory accumulators) give
    the mma.sync tiles' results: the same bf16 products summed in fp32 in
    another order, over several 128-row tiles and a partial one."""
    from ppf_gb300 import learned as PL

    torch = torch_cuda
    L = PL.lib()
    L.ppf_learned_clear_samples()
    s = learned_cases.synthetic(n=1000, seed=8)
    g = learned_cases.graph(s)
    k = _add(product_lib, s)
    w = _weights(5)
    wb = torch.tensor(w, device="cuda").to(torch.bfloat16).contiguous()
    E = len(g.lo)
    out = {}
    prev = L.ppf_learned_tensor_path(-1)
    try:
        for tc in (0, 1):
            L.ppf_learned_tensor_path(tc)
            a = np.zeros(E, np.float32)
            q = np.zeros(g.n, np.float32)
            assert L.ppf_learned_forward(k, wb.data_ptr(), a, q) == 0
            out[tc] = (a, q)
    finally:
        L.ppf_learned_tensor_path(prev)
    assert L.ppf_learned_tc_status() == 0
    (a0, q0), (a1, q1) = out[0], out[1]
    assert np.abs(q1 - q0).max() <= 5e-3 * max(1.0, np.abs(q0).max()), np.abs(q1 - q0).max()
    assert np.abs(a1 - a0).max() < 5e-3
    f = OL.forward(g, w)
    assert np.abs(q1 - f["q"])[g.free].max() <= 2e-2 * max(1.0, np.abs(f["q"]).max())
    # more 128-row tiles than resident CTAs: each CTA walks several tiles
    # through its double-buffered operand tiles
    L.ppf_learned_clear_samples()
    big = learned_cases.synthetic(n=50000, seed=9)
    k = _add(product_lib, big)
    E = int(big["f_off"][-1]) + int(big["d_off"][-1])
    try:
        for tc in (0, 1):
            L.ppf_learned_tensor_path(tc)
            a = np.zeros(E, np.float32)
            q = np.zeros(big["n"], np.float32)
            assert L.ppf_learned_forward(k, wb.data_ptr(), a, q) == 0
            out[tc] = (a, q)
    finally:
        L.ppf_learned_tensor_path(prev)
    assert L.ppf_learned_tc_status() == 0
    (a0, q0), (a1, q1) = out[0], out[1]
    assert np.abs(q1 - q0).max() <= 5e-3 * max(1.0, np.abs(q0).max()), np.abs(q1 - q0).max()
    assert np.abs(a1 - a0).max() < 5e-3
    L.ppf_learned_clear_samples()


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle(product_lib, torch_cuda):
    from ppf_gb300 import learned as PL

    torch = torch_cuda
    PL.lib().ppf_learned_clear_samples()
    s = learned_cases.synthetic(n=300, seed=6)
    g = learned_cases.graph(s)
    k = _add(product_lib, s)
    w = _weights(4)
    pr = learned_cases.probes(g.n, W=4, seed=9)
    wb = torch.tensor(w, device="cuda").to(torch.bfloat16).contiguous()
    pd = torch.tensor(pr, device="cuda").contiguous()
    grad = torch.empty(PL.N_WEIGHTS, dtype=torch.float32, device="cuda")
    loss = C.c_float()
    rc = PL.lib().ppf_learned_loss_grad(k, wb.data_ptr(), pd.data_ptr(), pr.shape[0],
                                        grad.data_ptr(), C.byref(loss),
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    L, go, _ = OL.loss_and_grad(g, w, pr)
    gg = grad.cpu().numpy()
    assert abs(loss.value - L) <= 1e-3 * max(1.0, abs(L)), (loss.value, L)
    rel = np.linalg.norm(gg - go) / np.linalg.norm(go)
    cos = float(gg @ go / (np.linalg.norm(gg) * np.linalg.norm(go)))
    assert rel < 3e-2 and cos > 0.999, (rel, cos)
    # every layer's block agrees on its own
    for name, v in OL.weight_views(go).items():
        vg = OL.weight_views(gg)[name]
        if np.linalg.norm(v) > 0:
            assert np.linalg.norm(vg - v) <= 5e-2 * np.linalg.norm(v), name


@pytest.mark.gpu
def test_gpu_training_lowers_the_loss(product_lib, torch_cuda):
    from ppf_gb300 import learned as PL
    from ppf_gb300 import scenes

    PL.lib().ppf_learned_clear_samples()
    sc, _ = scenes.stacked_sheets(side=32, sheets=4, seed=5)
    got = list(PL.collect(sc, 40, every=4, start=8))
    ids = [PL.add_sample(s) for s in got]
    assert len(ids) >= 6
    tr = PL.Trainer(ids[:-2], [s["n"] for s in got[:-2]], seed=0, lr=3e-3, probes=8)
    before = np.mean(PL.sample_loss(ids[-2:], tr.weights()))
    for it in range(150):
        tr.step(it % (len(ids) - 2))
    after = np.mean(PL.sample_loss(ids[-2:], tr.weights()))
    assert after < before - 0.01, (before, after)
    PL.lib().ppf_learned_clear_samples()


def _run(scene_fn, kind, steps, weights=None, motion=None):
    from ppf_gb300 import abi
    from ppf_gb300 import learned as PL
    from ppf_gb300.session import Session

    sc, m = scene_fn()
    if weights is not None:
        PL.use_weights(weights)
    s = Session(sc, pin_motion=motion or m)
    s.set_preconditioner(kind)
    iters = solves = fallbacks = 0
    ms = 0.0
    for _ in range(steps):
        r = s.step()
        assert r.success()
        st = s.stats()
        iters += st.pcg_iters_total
        solves += st.pcg_solves
        fallbacks += st.fallbacks
        ms += st.pcg_ms_total
    return iters, solves, fallbacks, ms, s


@pytest.mark.gpu
def test_learned_factor_matches_the_network(product_lib):
    """The solver's learned factor: G(i, i) = d_i C(i)^{-1} with d from the
    network on the same Newton system."""
    import step_scenes
    from ppf_gb300 import abi
    from ppf_gb300 import learned as PL
    from ppf_gb300.session import Session

    w = PL.load_weights()
    PL.use_weights(w)
    sc, _ = step_scenes.two_sheets()
    n = sc.vertex_count
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_LEARNED)
    sys_ = PL.capture_system(n)  # solves with the learned factor (forced)
    diag = np.zeros(9 * n, np.float32)
    PL.lib().ppf_debug_factor_diag(diag)
    g = learned_cases.graph(sys_)
    f = OL.forward(g, w)
    Gd = diag.reshape(n, 3, 3).transpose(0, 2, 1)
    want = f["d"][:, None, None] * g.cinv
    free = g.free
    err = np.abs(Gd[free] - want[free]).max() / np.abs(want[free]).max()
    assert err < 2e-2, err
    # the learned solve solves the system
    assert sys_["bj_iters"] > 0


@pytest.mark.gpu
def test_trained_network_gain_on_a_held_out_scene(product_lib):
    """The packaged network (trained on other seeds) against block-Jacobi and
    the first-order factor on a held-out stacked-sheets scene: PCG iterations
    and time over the same steps."""
    from ppf_gb300 import abi
    from ppf_gb300 import learned as PL
    from ppf_gb300 import scenes

    scene = lambda: scenes.stacked_sheets(side=64, sheets=8, seed=11)
    steps = 30
    bj = _run(scene, abi.PRECOND_BLOCK_JACOBI, steps)
    fo = _run(scene, abi.PRECOND_FIRST_ORDER, steps)
    le = _run(scene, abi.PRECOND_LEARNED, steps, weights=PL.load_weights())
    print(f"\nheld-out stacked sheets 64x8, {steps} steps: PCG iterations / solves / fallbacks / ms"
          f"\n  block-Jacobi {bj[:4]}\n  first-order  {fo[:4]}\n  learned      {le[:4]}")
    # iterations per solve of the factored solves (the fallback solves are
    # block-Jacobi and counted in pcg_iters_total as well)
    assert le[0] < bj[0], (le, bj)
    assert le[2] <= le[1] // 4, "the learned factor fell back on most solves"


@pytest.mark.gpu
def test_learned_trajectory_invariants(product_lib, oracle_lib):
    from oracle.binding import OracleSession
    from ppf_gb300 import abi, meshes, scenes
    from ppf_gb300 import learned as PL
    from ppf_gb300.session import Session

    PL.use_weights()
    sc, _ = scenes.cloth_sphere(24)
    s = Session(sc)
    s.set_preconditioner(abi.PRECOND_LEARNED)
    orc = OracleSession(sc)
    v, f = meshes.grid(24, 24)
    for step in range(40):
        r = s.step()
        assert r.success()
        if step % 8 == 7:
            x = s.positions()
            assert orc.intersection_free(x)
    assert s.stats().precond_kind == abi.PRECOND_LEARNED
