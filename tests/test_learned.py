"""Learned proposer: CPU oracle self-consistency, GPU kernels against the
oracle (forward, loss, gradients), and training reducing the loss."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_oracle  # noqa: E402


def _params(seed=0, scale=0.3):
    rng = np.random.default_rng(seed)
    p = {"w1": rng.normal(0, scale, (128, 56)).astype(np.float32), "w2": rng.normal(0, scale / 2, (128, 128)).astype(np.float32),
         "w3": rng.normal(0, scale, (5, 128)).astype(np.float32), "b1": rng.normal(0, 0.1, 128).astype(np.float32),
         "b2": rng.normal(0, 0.1, 128).astype(np.float32), "b3": rng.normal(0, 0.1, 5).astype(np.float32)}
    return p


def _batch(M=96, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (M, 56)).astype(np.float32)
    y = rng.normal(0, 1, M).astype(np.float32)
    b = rng.integers(0, 4, M).astype(np.int32)
    return x, y, b


def test_oracle_gradients_match_finite_differences():
    p = _params()
    x, y, b = _batch(16)
    loss, g, _ = mlp_oracle.loss_and_grads(x.astype(np.float64), y, b, p)
    # perturb biases (weights are bf16-rounded, so finite differences on them
    # would see the rounding steps)
    for k in ("b1", "b2", "b3"):
        for i in (0, 3):
            q = {kk: vv.copy() for kk, vv in p.items()}
            h = 1e-3
            q[k] = q[k].astype(np.float64)
            q[k][i] += h
            lp, _, _ = mlp_oracle.loss_and_grads(x.astype(np.float64), y, b, q)
            q[k][i] -= 2 * h
            lm, _, _ = mlp_oracle.loss_and_grads(x.astype(np.float64), y, b, q)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k][i]) <= 1e-5 + 1e-3 * abs(fd), (k, i, fd, g[k][i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.1415926], np.float32)
    r = mlp_oracle.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and abs(r[3] + 3.140625) < 1e-12


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_oracle():
    import torch
    import gcchem.learned as learned

    pr = learned.Proposer(0)
    p = _params()
    for k, v in p.items():
        pr.master[k] = torch.tensor(v, device=pr.dev)
    pr.bf = {k: pr.master[k].to(torch.bfloat16) for k in ("w1", "w2", "w3")}
    for k in pr.grad:
        pr.grad[k] = torch.zeros_like(pr.master[k])
    x, y, b = _batch(200)
    xt = torch.tensor(x, device=pr.dev)
    loss, a = pr.loss_grad(xt, torch.tensor(y, device=pr.dev), torch.tensor(b, device=pr.dev), w_ce=0.5)
    loss_ref, g_ref, f_ref = mlp_oracle.loss_and_grads(x.astype(np.float64), y, b, p, w_ce=0.5)
    out = a["out"].cpu().numpy()
    assert np.max(np.abs(out - f_ref["out"])) < 1e-3 * max(1.0, np.max(np.abs(f_ref["out"])))
    assert abs(loss.item() - loss_ref) < 1e-4 * max(1.0, loss_ref)
    for k in ("w1", "b1", "w2", "b2", "w3", "b3"):
        gg = pr.grad[k].cpu().numpy()
        ref = g_ref[k]
        scale = np.max(np.abs(ref)) + 1e-12
        assert np.max(np.abs(gg - ref)) / scale < 2e-3, k


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    import torch
    import gcchem.learned as learned

    rng = np.random.default_rng(5)
    M = 16384
    x = rng.normal(0, 1, (M, 56)).astype(np.float32)
    w = rng.normal(0, 1, 56)
    y = (x @ w / 8.0 + 0.3 * np.sin(x[:, 0])).astype(np.float32)
    b = np.digitize(x[:, 1] + x[:, 2], [-1.0, 0.0, 1.0]).astype(np.int32)
    pr = learned.Proposer(0, seed=3)
    t = lambda a: torch.tensor(a, device=pr.dev)
    hist = pr.train(t(x), t(y), t(b), epochs=5, batch=1024, lr=2e-3)
    # every epoch lowers the mean loss, and the last is a third below the first
    assert all(b < a for a, b in zip(hist, hist[1:])), hist
    assert hist[-1] < 0.67 * hist[0], hist


def test_makespan_model_of_the_queue():
    import gcchem.learned as learned

    work = np.r_[np.ones(30), 20.0]
    natural = np.arange(31)
    heavy_first = np.r_[30, np.arange(30)]
    # 4 slots: in grid order the heavy cell starts last and runs alone
    assert learned.makespan(work, natural, 4) == 7.0 + 20.0
    assert learned.makespan(work, heavy_first, 4) == 20.0
    # one slot per cell: the order cannot matter
    assert learned.makespan(work, natural, 64) == learned.makespan(work, heavy_first, 64) == 20.0


@pytest.mark.gpu
def test_gpu_propose_and_bin_order():
    """H0 = clamp(scale * exp(out[:,0])), bin = argmax(logits); the order is a
    permutation of the cells with the heaviest bin first."""
    import torch
    import gcchem.learned as learned

    pr = learned.Proposer(0, seed=4)
    rng = np.random.default_rng(8)
    M = 5000
    x = torch.tensor(rng.normal(0, 1, (M, 56)).astype(np.float32), device=pr.dev)
    pr.y_mean = 1.5
    h0, bins = pr.propose(x, hmin=1e-5, hmax=1200.0)
    out = pr.forward(x)["out"].cpu().numpy().astype(np.float64)
    ref_h = np.clip(pr.h0_scale * np.exp(pr.y_mean) * np.exp(out[:, 0]), 1e-5, 1200.0)
    assert np.allclose(h0.cpu().numpy(), ref_h, rtol=1e-6)
    assert np.array_equal(bins.cpu().numpy(), out[:, 1:].argmax(1))
    order = pr.bin_order(bins).cpu().numpy()
    b = bins.cpu().numpy()
    # heaviest bin first, ascending cells inside a bin (a stable sort)
    assert np.array_equal(order, np.argsort(-b, kind="stable"))
    assert np.array_equal(pr.last_counts.cpu().numpy(), np.bincount(b, minlength=4))
    big = torch.tensor(np.random.default_rng(2).integers(0, 4, 700_001).astype(np.int32), device=pr.dev)
    ob = pr.bin_order(big).cpu().numpy()
    assert np.array_equal(ob, np.argsort(-big.cpu().numpy(), kind="stable"))


@pytest.mark.gpu
def test_learned_step_c_abi_matches_python_plan():
    """gc_kpp_fullchem_step_learned (host and device memory) = the Python
    plan (features, MLP, proposals, stable bin order) + the binned step."""
    import torch
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned

    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    cp = learned.CProposer(prop)
    solver = capi.Solver(0, arith="fast", schedule="queue")
    n = 3000
    cells = inputs.grid_cells(20, 10, 15, seed=3)
    cells = {k: np.ascontiguousarray(cells[k][:, :n]) for k in ("met", "photol", "c")}
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    T = lambda a: torch.tensor(a, device=prop.dev).contiguous()

    def dev_arrays():
        return (T(cells["c"]), torch.zeros(n, dtype=torch.float64, device=prop.dev),
                torch.zeros((20, n), dtype=torch.int32, device=prop.dev),
                torch.zeros((20, n), dtype=torch.float64, device=prop.dev),
                torch.zeros(n, dtype=torch.int32, device=prop.dev))

    # Python plan + binned step
    c, hs, ist, rst, ierr = dev_arrays()
    met, ph = T(cells["met"]), T(cells["photol"])
    _, _, order = learned.plan(prop, met, ph, c, hstart=hs, hmax=600.0)
    nb = int(prop.last_counts[3].item())
    solver.fullchem_step(600.0, met, ph, c, T(atol), T(rtol), ic, rc, hs, ist, rst, ierr, order=order, nblock=nb)
    ref = [x.cpu().numpy() for x in (c, hs, ist, rst, ierr)]
    # C ABI, device memory
    c, hs, ist, rst, ierr = dev_arrays()
    _, nb_d = solver.fullchem_step_learned(cp.handle, 600.0, met, ph, c, T(atol), T(rtol), ic, rc, hs, ist, rst,
                                           ierr)
    got_d = [x.cpu().numpy() for x in (c, hs, ist, rst, ierr)]
    # C ABI, host memory
    ch = cells["c"].copy()
    hsh = np.zeros(n)
    isth = np.zeros((20, n), np.int32)
    rsth = np.zeros((20, n))
    ierrh = np.zeros(n, np.int32)
    _, nb_h = solver.fullchem_step_learned(cp.handle, 600.0, cells["met"], cells["photol"], ch, atol, rtol, ic, rc,
                                           hsh, isth, rsth, ierrh)
    # C ABI, page-locked host memory with padded rows (SM staging copies, the
    # PHOTOL rows that the rates and features read)
    ld = n + 5
    pinned = lambda a, dt=torch.float64: torch.zeros(a, dtype=dt).pin_memory()
    metp, php, cpn = pinned((18, ld)), pinned((200, ld)), pinned((cells["c"].shape[0], ld))
    metp[:, :n] = torch.from_numpy(cells["met"])
    php[:, :n] = torch.from_numpy(cells["photol"])
    cpn[:, :n] = torch.from_numpy(cells["c"])
    hsp, istp, rstp = pinned(n), pinned((20, ld), torch.int32), pinned((20, ld))
    ierrp = pinned(n, torch.int32)
    _, nb_p = solver.fullchem_step_learned(cp.handle, 600.0, metp[:, :n], php[:, :n], cpn[:, :n], atol, rtol, ic, rc,
                                           hsp, istp[:, :n], rstp[:, :n], ierrp)
    got_p = [x.numpy() for x in (cpn[:, :n], hsp, istp[:, :n], rstp[:, :n], ierrp)]
    assert nb_d == nb_h == nb_p == nb
    for got in (got_d, [ch, hsh, isth, rsth, ierrh], got_p):
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    assert np.all(cpn[:, n:].numpy() == 0) and np.all(istp[:, n:].numpy() == 0)  # padding untouched
    cp.close()


@pytest.mark.gpu
def test_learned_steps_capture_in_a_cuda_graph():
    """Two learned chemistry steps (plan + binned step + hand-over) captured in
    one CUDA graph give the results of two synchronous learned steps."""
    import torch
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned

    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    cp = learned.CProposer(prop)
    solver = capi.Solver(0, arith="fast", schedule="queue", block=64)
    solver.set(evict_after=2, cell_block=128)
    cells = inputs.grid_cells(20, 10, 16, seed=6)
    n = cells["c"].shape[1]
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    dev = prop.dev
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    met, ph, c0, at, rt = T(cells["met"]), T(cells["photol"]), T(cells["c"]), T(atol), T(rtol)
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)
    c, hs, ist, rst, ierr = c0.clone(), z(n), z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)

    def steps(stream=None):
        for _ in range(2):
            solver.fullchem_step_learned(cp.handle, 600.0, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr,
                                         stream=stream)

    steps()
    torch.cuda.synchronize()
    ref = [x.cpu().numpy() for x in (c, hs, ist, rst, ierr)]
    solver.set(async_steps=True)
    c.copy_(c0)
    hs.zero_()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        steps(stream=torch.cuda.current_stream().cuda_stream)
    c.copy_(c0)
    hs.zero_()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip([x.cpu().numpy() for x in (c, hs, ist, rst, ierr)], ref):
        assert np.array_equal(a, b)
    solver.set(async_steps=False, evict_after=0)
    cp.close()
