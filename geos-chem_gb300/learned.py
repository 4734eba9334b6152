"""Learned step-size / stiffness proposer: host side.

A 56 -> 128 -> 128 -> 5 MLP (GELU), BF16 weights with FP32 master copies,
trained on the GPU by this package's own kernels (csrc/kpp_mlp.cu through
include/gckpp_gb300_mlp.h).  Inputs are a cell's state: log T, log P, log
H2O mixing ratio, cos SZA, 20 log J-values and 32 log key-species mixing
ratios, normalised.  Outputs: log of a proposed initial step size H0 and
logits of 4 stiffness bins.

Training targets come from plain GPU integrations (``collect``): the
integrator's own next-step prediction at the end of the step, RSTATUS(3)
(Hnew, what GEOS-Chem carries to the next step as KPPHvalue), and the
quartile bin of the step count ISTATUS(3).  The proposal seeds RCNTRL(3)
(scaled down by ``h0_scale``) and orders the persistent solver's queue by
predicted bin, heaviest first; error-controlled Rosenbrock still decides
every step.

torch tensors are used only as device allocations and streams.
"""
import ctypes
import json
import os

import numpy as np

from . import capi, inputs, mechanism

NFEAT, HID, NOUT, NJ, NSPC, NBIN = 56, 128, 5, 20, 32, 4
# largest proposed H0 [s] of a cold-started cell: DeltaMin * FacMax**8 =
# 1e-5 * 6**8 = 16.8 s, the step the plain method's cold start reaches at its
# ninth step when no step is limited by the error.  A first step far beyond
# the sizes of that ramp leaves the integration's last steps larger than the
# plain method's and its error against an RTOL 1e-8 integration larger; from
# this cap on the remaining steps follow the ramp, so the error stays at the
# plain method's level while the ramp's first eight steps are skipped.
H0_CAP = 1.0e-5 * 6.0 ** 8
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "proposer_fullchem.npz")
BIN_EDGES = (2, 4, 16)  # Rosenbrock steps per chemistry step: 1 | 2-3 | 4-15 | >= 16

J_SPECIES = ["NO2", "O3", "O3", "HNO2", "H2O2", "HNO3", "HNO4", "NO3", "NO3", "N2O5", "CH2O", "CH2O", "MP",
             "Cl2", "Br2", "BrO", "ClNO3", "HOBr", "MGLY", "ALD2"]
KEY_SPECIES = ["O3", "NO", "NO2", "NO3", "N2O5", "HNO3", "HNO2", "HNO4", "OH", "HO2", "H2O2", "CO", "CH4", "CH2O",
               "MP", "PAN", "ISOP", "ALD2", "ACET", "SO2", "DMS", "Cl", "ClO", "HCl", "HOCl", "Br", "BrO", "HBr",
               "HOBr", "IO", "C2H6", "MVK"]


def feature_rows(ir=None):
    """(PHOTOL rows [20], species rows [32]) of the feature vector."""
    ir = ir or mechanism.load_ir()
    slots = inputs.photolysis_slots(ir)
    by_sp = {}
    for slot, sp in sorted(slots.items()):
        by_sp.setdefault(sp, []).append(slot)
    used = {}
    jrows = []
    for sp in J_SPECIES:
        k = used.get(sp, 0)
        jrows.append(by_sp[sp][min(k, len(by_sp[sp]) - 1)])
        used[sp] = k + 1
    srows = [ir["species"].index(s) for s in KEY_SPECIES]
    assert len(jrows) == NJ and len(srows) == NSPC
    return np.array(jrows, np.int32), np.array(srows, np.int32)


def _lib():
    lib = capi.load_library()
    vp, i32, i64, f32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float, ctypes.c_double
    lib.gc_mlp_features.argtypes = [i32, vp, i64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp]
    lib.gc_mlp_forward.argtypes = [i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gc_mlp_loss.argtypes = [i32, vp, vp, vp, f32, vp, vp, vp]
    lib.gc_mlp_backward.argtypes = [i32] + [vp] * 16 + [vp]
    lib.gc_mlp_adam.argtypes = [i32, vp, vp, vp, vp, vp, f32, f32, f32, f32, i32, vp]
    lib.gc_mlp_propose.argtypes = [i32, vp, f64, f64, f64, vp, vp, i32, vp]
    lib.gc_mlp_bin_order.argtypes = [i32, vp, vp, vp, vp, vp]
    lib.gc_mlp_bin_order_scratch.argtypes = [i32]
    return lib


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (%d)" % (what, rc))


class Proposer:
    """MLP parameters, optimiser state and the GPU kernels that use them."""

    def __init__(self, device=0, seed=0, h0_scale=0.5):
        import torch

        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.lib = _lib()
        rng = np.random.default_rng(seed)
        shapes = {"w1": (HID, NFEAT), "w2": (HID, HID), "w3": (NOUT, HID)}
        self.master = {}
        for k, (n, m) in shapes.items():
            w = rng.normal(0.0, np.sqrt(2.0 / (n + m)), (n, m)).astype(np.float32)
            self.master[k] = torch.tensor(w, device=self.dev)
        for k, n in (("b1", HID), ("b2", HID), ("b3", NOUT)):
            self.master[k] = torch.zeros(n, dtype=torch.float32, device=self.dev)
        self.bf = {k: self.master[k].to(torch.bfloat16) for k in ("w1", "w2", "w3")}
        self.grad = {k: torch.zeros_like(v) for k, v in self.master.items()}
        self.m1 = {k: torch.zeros_like(v) for k, v in self.master.items()}
        self.m2 = {k: torch.zeros_like(v) for k, v in self.master.items()}
        self.step_count = 0
        jrows, srows = feature_rows()
        self.jrows = torch.tensor(jrows, device=self.dev)
        self.srows = torch.tensor(srows, device=self.dev)
        self.mean = torch.zeros(NFEAT, dtype=torch.float64, device=self.dev)
        self.inv_std = torch.ones(NFEAT, dtype=torch.float64, device=self.dev)
        self.h0_scale = h0_scale
        self.h0_cap = H0_CAP
        self.bin_edges = [0.0, 0.0, 0.0]
        self.y_mean = 0.0

    # -- features -----------------------------------------------------------
    def features(self, met, photol, c, suncos=None, stream=None, raw=False):
        """Network inputs of every cell ([ncell, 56] float32); raw=True skips
        the normalisation (training data)."""
        t = self.torch
        n = c.shape[1]
        x = t.empty((n, NFEAT), dtype=t.float32, device=self.dev)
        mean, inv_std = self.mean, self.inv_std
        if raw:
            mean = t.zeros(NFEAT, dtype=t.float64, device=self.dev)
            inv_std = t.ones(NFEAT, dtype=t.float64, device=self.dev)
        _check(self.lib.gc_mlp_features(n, _p(met), met.stride(0), _p(photol), photol.stride(0), _p(c), c.stride(0),
                                        _p(suncos), _p(self.jrows), _p(self.srows), _p(mean), _p(inv_std),
                                        _p(x), stream), "features")
        return x

    def fit_normalisation(self, met, photol, c, suncos=None):
        self.mean.zero_()
        self.inv_std.fill_(1.0)
        x = self.features(met, photol, c, suncos).double()
        self.mean = x.mean(0).contiguous()
        self.inv_std = (1.0 / x.std(0).clamp_min(1e-6)).contiguous()

    # -- forward / backward -------------------------------------------------
    def _acts(self, M, train):
        t = self.torch
        f = lambda *s: t.empty(s, dtype=t.float32, device=self.dev)
        return {"z1": f(M, HID) if train else None, "h1": f(M, HID), "z2": f(M, HID) if train else None,
                "h2": f(M, HID), "out": f(M, NOUT)}

    def forward(self, x, train=False, stream=None):
        M = x.shape[0]
        a = self._acts(M, train)
        m, b = self.master, self.bf
        _check(self.lib.gc_mlp_forward(M, _p(x), _p(b["w1"]), _p(m["b1"]), _p(b["w2"]), _p(m["b2"]), _p(b["w3"]),
                                       _p(m["b3"]), _p(a["z1"]), _p(a["h1"]), _p(a["z2"]), _p(a["h2"]), _p(a["out"]),
                                       stream), "forward")
        return a

    def loss_grad(self, x, y_h, y_bin, w_ce=0.5):
        """Forward + loss + backward; gradients accumulate into self.grad."""
        t = self.torch
        M = x.shape[0]
        a = self.forward(x, train=True)
        dout = t.empty((M, NOUT), dtype=t.float32, device=self.dev)
        loss = t.zeros(1, dtype=t.float32, device=self.dev)
        _check(self.lib.gc_mlp_loss(M, _p(a["out"]), _p(y_h), _p(y_bin), float(w_ce), _p(dout), _p(loss), None),
               "loss")
        scratch = t.empty(M * (NOUT + 4 * HID), dtype=t.float32, device=self.dev)
        g, b = self.grad, self.bf
        _check(self.lib.gc_mlp_backward(M, _p(x), _p(b["w1"]), _p(b["w2"]), _p(b["w3"]), _p(a["z1"]), _p(a["h1"]),
                                        _p(a["z2"]), _p(a["h2"]), _p(dout), _p(g["w1"]), _p(g["b1"]), _p(g["w2"]),
                                        _p(g["b2"]), _p(g["w3"]), _p(g["b3"]), _p(scratch), None), "backward")
        return loss, a

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for k, w in self.master.items():
            _check(self.lib.gc_mlp_adam(w.numel(), _p(w), _p(self.bf.get(k)), _p(self.grad[k]), _p(self.m1[k]),
                                        _p(self.m2[k]), lr, b1, b2, eps, self.step_count, None), "adam")

    # -- training -------------------------------------------------------------
    def fit_targets(self, hnew, steps, edges=BIN_EDGES):
        """Centre of log(Hnew) and the step-count edges of the 4 stiffness
        bins (bin b holds cells with edges[b-1] <= steps < edges[b]).  The
        last bin is the few cells that need tens of steps, the ones the
        block-per-cell kernel takes."""
        t = self.torch
        self.y_mean = float(t.log(hnew.double().clamp_min(1e-10)).mean().item())
        self.bin_edges = [float(v) for v in edges]

    def targets(self, hnew, steps):
        """log(Hnew) (centred) and the stiffness bin of each row."""
        t = self.torch
        h = (t.log(hnew.double().clamp_min(1e-10)) - self.y_mean).float()
        e = t.tensor(self.bin_edges, dtype=t.float64, device=steps.device)
        b = t.bucketize(steps.double(), e, right=True).int()
        return h.contiguous(), b.contiguous()

    def normalise(self, x_raw):
        """Rows of raw features -> the network's inputs (what the features
        kernel produces with this normalisation)."""
        return ((x_raw.double() - self.mean) * self.inv_std).float().contiguous()

    def fit_normalisation_rows(self, x_raw):
        x = x_raw.double()
        self.mean = x.mean(0).contiguous()
        self.inv_std = (1.0 / x.std(0).clamp_min(1e-6)).contiguous()

    def train(self, x, y_h, y_bin, epochs=4, batch=4096, lr=2e-3, w_ce=0.5, seed=0, log=None):
        t = self.torch
        n = x.shape[0]
        gen = t.Generator(device=self.dev)
        gen.manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = t.randperm(n, device=self.dev, generator=gen)
            tot = t.zeros(1, dtype=t.float32, device=self.dev)
            nb = 0
            lr_ep = lr * (0.5 ** ep)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                loss, _ = self.loss_grad(x[idx].contiguous(), y_h[idx].contiguous(), y_bin[idx].contiguous(), w_ce)
                self.adam_step(lr_ep)
                tot += loss
                nb += 1
            hist.append(float((tot / max(nb, 1)).item()))
            if log:
                log("epoch %d loss %.4f" % (ep, hist[-1]))
        return hist

    # -- inference ------------------------------------------------------------
    def propose(self, x, hmin=1e-5, hmax=1.0e9, stream=None, h0=None):
        """H0 proposals and stiffness bins.  If `h0` is given, it is filled in
        place where it is not positive (cells without a KPPHvalue)."""
        t = self.torch
        M = x.shape[0]
        a = self.forward(x, stream=stream)
        keep = h0 is not None
        if h0 is None:
            h0 = t.empty(M, dtype=t.float64, device=self.dev)
        b = t.empty(M, dtype=t.int32, device=self.dev)
        # the network's log-H output is centred on y_mean: fold exp(y_mean) into the scale
        scale = float(self.h0_scale * np.exp(self.y_mean))
        _check(self.lib.gc_mlp_propose(M, _p(a["out"]), scale, hmin, hmax, _p(h0), _p(b), int(keep), stream),
               "propose")
        return h0, b

    def bin_order(self, bins, stream=None):
        t = self.torch
        M = bins.shape[0]
        order = t.empty(M, dtype=t.int32, device=self.dev)
        counts = t.empty(NBIN, dtype=t.int32, device=self.dev)
        scratch = t.empty(max(NBIN, self.lib.gc_mlp_bin_order_scratch(M)), dtype=t.int32, device=self.dev)
        _check(self.lib.gc_mlp_bin_order(M, _p(bins), _p(counts), _p(scratch), _p(order), stream), "bin_order")
        self.last_counts = counts
        return order

    # -- persistence -----------------------------------------------------------
    def state(self):
        d = {k: v.cpu().numpy() for k, v in self.master.items()}
        d.update(mean=self.mean.cpu().numpy(), inv_std=self.inv_std.cpu().numpy())
        d["meta"] = np.array(json.dumps({"h0_scale": self.h0_scale, "bin_edges": self.bin_edges,
                                         "y_mean": self.y_mean}))
        return d

    def load_state(self, d):
        t = self.torch
        for k in ("w1", "w2", "w3", "b1", "b2", "b3"):
            self.master[k] = t.tensor(d[k], dtype=t.float32, device=self.dev)
        self.bf = {k: self.master[k].to(t.bfloat16) for k in ("w1", "w2", "w3")}
        self.mean = t.tensor(d["mean"], dtype=t.float64, device=self.dev)
        self.inv_std = t.tensor(d["inv_std"], dtype=t.float64, device=self.dev)
        meta = json.loads(str(d["meta"]))
        self.h0_scale, self.bin_edges, self.y_mean = meta["h0_scale"], meta["bin_edges"], meta["y_mean"]


# -- training data from plain GPU runs -------------------------------------------
def device_cells(cells, dev):
    """The met / photol / C arrays of a cell set as contiguous CUDA tensors."""
    import torch

    return {k: torch.tensor(cells[k], dtype=torch.float64, device=dev).contiguous() for k in ("met", "photol", "c")}


def collect(solver, prop, cells, dt=1200.0, nsteps=2, spinup=86400.0, log=None):
    """Plain GPU chemistry steps over a cell set, as Do_FullChem runs them:
    a spin-up step of `spinup` seconds, then `nsteps` steps of `dt` seconds
    with the KPPHvalue chain.  Returns per cell-step rows: raw features at the
    start of the step, Hnew (RSTATUS(3)) and the step count (ISTATUS(3)) at
    its end -- the (state, accepted step size, step count) training pairs."""
    import torch

    d = device_cells(cells, prop.dev)
    n = d["c"].shape[1]
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    at = torch.tensor(atol, device=prop.dev)
    rt = torch.tensor(rtol, device=prop.dev)
    hs = torch.zeros(n, dtype=torch.float64, device=prop.dev)
    ist = torch.zeros((20, n), dtype=torch.int32, device=prop.dev)
    rst = torch.zeros((20, n), dtype=torch.float64, device=prop.dev)
    ierr = torch.zeros(n, dtype=torch.int32, device=prop.dev)
    if spinup > 0:
        solver.fullchem_step(spinup, d["met"], d["photol"], d["c"], at, rt, ic, rc, hs, ist, rst, ierr)
    xs, hn, st = [], [], []
    for k in range(nsteps):
        xs.append(prop.features(d["met"], d["photol"], d["c"], raw=True))
        solver.fullchem_step(dt, d["met"], d["photol"], d["c"], at, rt, ic, rc, hs, ist, rst, ierr)
        hn.append(rst[2].clone())
        st.append(ist[2].clone())
        if log:
            log("step %d: mean steps %.2f" % (k, st[-1].double().mean().item()))
    torch.cuda.synchronize()
    return {"x": torch.cat(xs), "hnew": torch.cat(hn), "steps": torch.cat(st)}


def fit(prop, data, epochs=6, batch=4096, lr=2e-3, w_ce=0.5, edges=BIN_EDGES, seed=0, log=None):
    """Normalisation, targets and training of `prop` on collected rows."""
    prop.fit_normalisation_rows(data["x"])
    prop.fit_targets(data["hnew"], data["steps"], edges)
    x = prop.normalise(data["x"])
    y_h, y_b = prop.targets(data["hnew"], data["steps"])
    return prop.train(x, y_h, y_b, epochs=epochs, batch=batch, lr=lr, w_ce=w_ce, seed=seed, log=log)


def makespan(work, order, nslot):
    """Completion time of a list schedule: `nslot` workers take cells in
    `order`, each as soon as it is free; cell i costs work[i].  Models the
    persistent queue kernel, whose slots claim the next cell when theirs is
    done."""
    import heapq

    work = np.asarray(work, dtype=np.float64)
    order = np.asarray(order)
    k = min(nslot, len(order))
    free = list(work[order[:k]])
    heapq.heapify(free)
    for c in order[k:]:
        t = heapq.heappop(free)
        heapq.heappush(free, t + work[c])
    return max(free) if free else 0.0


def evaluate(prop, data):
    """Held-out quality: log-H RMSE, bin accuracy and, per true bin, how
    many cells the network puts there."""
    t = prop.torch
    x = prop.normalise(data["x"])
    a = prop.forward(x)
    y_h, y_b = prop.targets(data["hnew"], data["steps"])
    out = a["out"]
    rmse = float(t.sqrt(((out[:, 0] - y_h) ** 2).mean()).item())
    pred_b = out[:, 1:].argmax(1).int()
    acc = float((pred_b == y_b).double().mean().item())
    per_bin = {}
    for b in range(NBIN):
        sel = y_b == b
        n = int(sel.sum().item())
        per_bin[str(b)] = {"cells": n, "recall": float((pred_b[sel] == b).double().mean().item()) if n else None,
                           "predicted": int((pred_b == b).sum().item())}
    return {"logh_rmse": rmse, "bin_accuracy": acc, "bins": per_bin, "edges": prop.bin_edges}


class CProposer:
    """A Proposer's weights on the device behind the C ABI (gc_kpp_proposer),
    for Solver.fullchem_step_learned."""

    def __init__(self, prop, device=0):
        lib = capi.load_library()
        vp, i32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.gc_kpp_proposer_create.argtypes = [i32] + [vp] * 10 + [f64, ctypes.POINTER(vp)]
        lib.gc_kpp_proposer_destroy.argtypes = [vp]
        self.lib = lib
        host = lambda t, dt: np.ascontiguousarray(t.detach().cpu().numpy(), dtype=dt)
        arrs = [host(prop.master[k], np.float32) for k in ("w1", "b1", "w2", "b2", "w3", "b3")]
        arrs += [host(prop.mean, np.float64), host(prop.inv_std, np.float64), host(prop.jrows, np.int32),
                 host(prop.srows, np.int32)]
        self._keep = arrs
        self.handle = ctypes.c_void_p()
        scale = float(prop.h0_scale * np.exp(prop.y_mean))
        rc = lib.gc_kpp_proposer_create(device, *[a.ctypes.data_as(vp) for a in arrs], scale,
                                        ctypes.byref(self.handle))
        if rc != 0:
            raise capi.GcKppError(rc, lib.gc_kpp_last_error().decode())
        lib.gc_kpp_proposer_set_h0_cap.argtypes = [vp, f64]
        rc = lib.gc_kpp_proposer_set_h0_cap(self.handle, float(prop.h0_cap or 0.0))
        if rc != 0:
            raise capi.GcKppError(rc, lib.gc_kpp_last_error().decode())

    def close(self):
        if self.handle:
            self.lib.gc_kpp_proposer_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


PLAN_LAUNCHES = 8  # features 1, forward 3, propose 1, bin order 3


def plan(prop, met, photol, c, stream=None, hstart=None, hmax=1.0e9):
    """The learned part of a chemistry step, on the GPU: features of every
    cell, the MLP, H0 proposals (at most min(hmax, prop.h0_cap)) and
    stiffness bins, and the queue order (heaviest predicted bin first).
    Launches PLAN_LAUNCHES kernels.  The per-bin cell counts are left in
    ``prop.last_counts`` (device).  With `hstart` (the KPPHvalue array),
    proposals fill it in place where it is not positive and it is returned
    as H0."""
    x = prop.features(met, photol, c, stream=stream)
    if prop.h0_cap:
        hmax = min(hmax, prop.h0_cap)
    h0, bins = prop.propose(x, stream=stream, h0=hstart, hmax=hmax)
    order = prop.bin_order(bins, stream=stream)
    return h0, bins, order
