"""Learned closure of the micro cells (config 5 form).

A learned cell carries one unknown, the mean water content theta of its
inclusion's interior nodes.  With H_c the macro head at the cell centre and
theta_B(H_c) the water content of material B at that head, the closure is a
relaxation in water content,

    exchange inflow      Q           = kQ (theta_B(H_c) - theta)
    interior water rate  d theta/dt  = kT (theta_B(H_c) - theta),

smooth in every input and linear in theta.

and the network predicts the coefficients from six inputs -- the macro
head, its rates over the last three accepted steps, theta and h(theta):

    kQ = exp(y1),   kT = exp(y1 - y2) / (s^2 A_int)

(s the cell's inclusion scale, A_int the template's interior CV area, so
both outputs are free of the cell size; y2 is the log of the ratio of the
exchange inflow to the interior water rate s^2 A_int dtheta/dt, which the
plain method keeps near a constant, so that the closure's water balance
rests on one well-learned output instead of on two independent ones).  The coefficients are evaluated
once per accepted step by the BF16 tensor-core network and held fixed
during the step, so G stays smooth in FP64 and the finite-difference
Jacobian of EXPREM sees the exact linearisation of the closure.

After every step an a-posteriori indicator compares the inflow the held
coefficients gave with the one the network gives at the new state,
|kQ' - kQ| |d| / max(kQ' |d|, q_floor), d = theta_B(H_c) - theta (once a
cell has the three-step head history its rate inputs need), and flags
inputs outside
the training range; flagged cells fall back to their micro meshes and the
plain FP64 cell kernel for the rest of the run.

Training data are logged from plain-method runs: after every accepted step
the per-cell summary (tsr_cell_summary) gives H_c, theta, d theta/dt and Q
of every cell, from which the inputs and the targets
y1 = log(Q / d), y2 = log(Q / (s^2 A_int d theta/dt)) are formed where both
ratios are positive.
"""
import ctypes as C
import time

import numpy as np

from . import capi
from . import problem as P
from .capi import check, ptr

N_FEAT = 6


# ---- data ------------------------------------------------------------------
def interior_area(p):
    """s^2 A_int of every cell (inclusion interior CV area, physical units)."""
    lib_mesh = p.micro
    mn = lib_mesh.no_nodes
    cv = capi.as_array(lib_mesh.CV_area, mn, np.float64)
    bnd = capi.as_array(lib_mesh.boundary_nodes, mn, np.int32)
    a = float(cv[bnd != 1].sum())
    s = p._scale if p._scale is not None else np.ones(p.Ne)
    return (s * s) * a


def theta_of(h, soil):
    """water content of a van Genuchten material (dict) at head h"""
    h = np.asarray(h, dtype=np.float64)
    m = 1.0 - 1.0 / soil["n"]
    Se = np.where(h < 0.0, (1.0 + (soil["alpha"] * np.abs(h)) ** soil["n"]) ** (-m), 1.0)
    return soil["thetar"] + (soil["thetas"] - soil["thetar"]) * Se


def features(Hc, hist, t, th, hb):
    """Inputs of the network (before standardisation).  hist: (n, 3) macro
    heads of the last three accepted states (NaN where missing), t: the
    four times (current first)."""
    n = Hc.size
    r = np.zeros((n, 3))
    prev = np.column_stack([Hc, hist])
    for i in range(3):
        dt = t[i] - t[i + 1]
        ok = np.isfinite(prev[:, i + 1])
        if dt > 0:
            r[ok, i] = (prev[ok, i] - prev[ok, i + 1]) / dt
    f = np.empty((n, N_FEAT))
    f[:, 0] = np.log(np.maximum(-Hc, 1e-6))
    f[:, 1:4] = np.arcsinh(r)
    f[:, 4] = th
    f[:, 5] = np.log(np.maximum(-hb, 1e-6))
    return f


def log_plain_run(p, max_steps=100000, cell_stride=1, time_limit=None, t_stop=None):
    """Run the plain method on the GPU to p.tend (or t_stop) and return, for
    every accepted step, (t, summary[Ne, 5]) of every cell_stride-th cell."""
    ctx = P.Context(p)
    lib = ctx.lib
    check(lib.tsr_exprem_load(ctx.h, ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    t = C.c_double(0.0)
    out = np.empty(5 * p.Ne)
    tspan = np.array([0.0])
    logs = []
    t0 = time.perf_counter()
    check(lib.tsr_cell_summary(ctx.h, None, ptr(out)), "summary")
    logs.append((0.0, out.reshape(p.Ne, 5)[::cell_stride].astype(np.float32)))
    t_end = p.tend if t_stop is None else min(p.tend, t_stop)
    while t.value < t_end and len(logs) <= max_steps:
        check(lib.tsr_exprem_advance(ctx.h, t_end, ptr(tspan), None, C.byref(p.options), C.byref(st),
                                     C.byref(t)), "advance")
        check(lib.tsr_cell_summary(ctx.h, None, ptr(out)), "summary")
        logs.append((t.value, out.reshape(p.Ne, 5)[::cell_stride].astype(np.float32)))
        if time_limit and time.perf_counter() - t0 > time_limit:
            break
    ctx.close()
    return logs


def samples(p, logs, cell_stride=1, min_gap=1e-12, skip=0):
    """(X [n, 8] float32 with 6 inputs, Y [n, 2] float32 targets) from a
    log, leaving out the first `skip` steps."""
    aint = interior_area(p)[::cell_stride]
    Xs, Ys = [], []
    for n in range(max(1, skip), len(logs)):
        t = [logs[n - i][0] if n - i >= 0 else np.nan for i in range(4)]
        S = logs[n][1].astype(np.float64)
        Hc, th, rate, Q, hb = S[:, 0], S[:, 1], S[:, 2], S[:, 3], S[:, 4]
        hist = np.full((Hc.size, 3), np.nan)
        for i in range(3):
            if n - 1 - i >= 0:
                hist[:, i] = logs[n - 1 - i][1][:, 0]
        tt = [x if np.isfinite(x) else -1e30 for x in t]
        f = features(Hc, hist, tt, th, hb)
        d = theta_of(Hc, p.soilB_dict) - th
        ok = np.abs(d) > min_gap
        ok[ok] = (Q[ok] / d[ok] > 0) & (rate[ok] / d[ok] > 0)
        y1 = np.log(Q[ok] / d[ok])
        # second target: log of the exchange-to-interior-rate ratio
        # Q / (s^2 A_int dtheta/dt), so that the closure's water balance
        # depends on this (nearly constant) ratio alone
        y2 = y1 - np.log(aint[ok] * rate[ok] / d[ok])
        X = np.zeros((ok.sum(), 8), dtype=np.float32)
        X[:, :N_FEAT] = f[ok]
        Xs.append(X)
        Ys.append(np.column_stack([y1, y2]).astype(np.float32))
    return np.concatenate(Xs), np.concatenate(Ys)


# ---- model -------------------------------------------------------------------
class ClosureModel:
    """Network parameters and the standardisation of inputs and outputs."""

    def __init__(self, params, fmu, fsd, ymu, ysd, zlo, zhi, params2=None):
        self.params = np.ascontiguousarray(params, dtype=np.float32)
        # ensemble partner: the same network trained from another seed
        self.params2 = None if params2 is None else np.ascontiguousarray(params2, dtype=np.float32)
        self.fmu, self.fsd = np.asarray(fmu, float), np.asarray(fsd, float)
        self.ymu, self.ysd = np.asarray(ymu, float), np.asarray(ysd, float)
        self.zlo, self.zhi = np.asarray(zlo, np.float32), np.asarray(zhi, np.float32)

    def norm(self):
        return np.ascontiguousarray(np.concatenate([self.fmu, self.fsd, self.ymu, self.ysd]))

    def zrange(self):
        return np.ascontiguousarray(np.concatenate([self.zlo, self.zhi]), dtype=np.float32)

    def save(self, path):
        extra = {} if self.params2 is None else {"params2": self.params2}
        np.savez(path, params=self.params, fmu=self.fmu, fsd=self.fsd, ymu=self.ymu, ysd=self.ysd,
                 zlo=self.zlo, zhi=self.zhi, **extra)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        return cls(d["params"], d["fmu"], d["fsd"], d["ymu"], d["ysd"], d["zlo"], d["zhi"],
                   d["params2"] if "params2" in d.files else None)


# parameter block of include/tsr_capi.h: (n_out, n_in) per layer, W then b
LAYERS = [(64, 16), (64, 64), (64, 64), (64, 64), (8, 64)]


def init_params(seed):
    """Seeded initial parameters: uniform(+-1/sqrt(fan_in)) weights on the
    real inputs and outputs, zero biases and padding."""
    rng = np.random.default_rng(seed)
    out = []
    for li, (no, ni) in enumerate(LAYERS):
        fan_in = N_FEAT if li == 0 else ni
        W = rng.uniform(-1.0, 1.0, size=(no, ni)) / np.sqrt(fan_in)
        if li == 0:
            W[:, N_FEAT:] = 0.0
        if li == len(LAYERS) - 1:
            W[2:, :] = 0.0
        out += [W.ravel(), np.zeros(no)]
    return np.concatenate(out).astype(np.float32)


class Mlp:
    """The tensor-core network (tsr_mlp)."""

    def __init__(self, params=None):
        self.lib = capi.load()
        self.h = self.lib.tsr_mlp_create()
        if not self.h:
            raise capi.TsrError(1, "tsr_mlp_create")
        self.n_params = self.lib.tsr_mlp_num_params()
        if params is not None:
            self.set_params(params)

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.lib.tsr_mlp_set_params(self.h, p.ctypes.data_as(capi.fp)), "tsr_mlp_set_params")

    def get_params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        check(self.lib.tsr_mlp_get_params(self.h, p.ctypes.data_as(capi.fp)), "tsr_mlp_get_params")
        return p

    def forward(self, x, fused=True):
        """fused: True (mma.sync, activations in registers), False (the
        layer-by-layer training path) or "tcgen05" (tensor memory)."""
        if fused == "tcgen05":
            fused = 2
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], 2), dtype=np.float32)
        check(self.lib.tsr_mlp_forward(self.h, x.ctypes.data_as(capi.fp), x.shape[0],
                                       y.ctypes.data_as(capi.fp), int(fused)), "tsr_mlp_forward")
        return y

    def grad(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        check(self.lib.tsr_mlp_grad(self.h, x.ctypes.data_as(capi.fp), y.ctypes.data_as(capi.fp),
                                    x.shape[0], C.byref(loss), g.ctypes.data_as(capi.fp)), "tsr_mlp_grad")
        return loss.value, g

    def train(self, X, Y, epochs=8, batch=4096, lr=2e-3, wd=1e-4, seed=1001):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        check(self.lib.tsr_mlp_set_data(self.h, X.ctypes.data_as(capi.fp), Y.ctypes.data_as(capi.fp),
                                        X.shape[0]), "tsr_mlp_set_data")
        hist = np.zeros(epochs, dtype=np.float32)
        check(self.lib.tsr_mlp_train(self.h, epochs, batch, lr, wd, seed, hist.ctypes.data_as(capi.fp)),
              "tsr_mlp_train")
        return hist

    def close(self):
        if self.h:
            self.lib.tsr_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def standardise(X, Y, margin=0.25):
    """Standardisation of a training set and the accepted feature range
    (training min/max of the standardised inputs widened by margin)."""
    f = X[:, :N_FEAT].astype(np.float64)
    fmu, fsd = f.mean(0), f.std(0)
    fsd[fsd < 1e-12] = 1.0
    ymu, ysd = Y.mean(0).astype(np.float64), Y.std(0).astype(np.float64)
    ysd[ysd < 1e-12] = 1.0
    Z = (f - fmu) / fsd
    zlo, zhi = Z.min(0) - margin, Z.max(0) + margin
    Xs = np.zeros_like(X)
    Xs[:, :N_FEAT] = Z.astype(np.float32)
    Ys = ((Y - ymu) / ysd).astype(np.float32)
    return Xs, Ys, (fmu, fsd, ymu, ysd, zlo, zhi)


def train_model(X, Y, epochs=8, batch=4096, lr=2e-3, wd=1e-4, seed=1001, holdout=0.05, ensemble=True):
    """Train the network on the GPU (and, with ensemble, a second one from
    seed + 1000 on the same standardised data: its disagreement with the
    first is the closure's error indicator); returns (ClosureModel, epoch
    losses of the first network, held-out relative errors of kQ and kT)."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(X.shape[0])
    nh = int(holdout * X.shape[0])
    Xs, Ys, st = standardise(X[perm[nh:]], Y[perm[nh:]])
    net = Mlp(init_params(seed))
    hist = net.train(Xs, Ys, epochs=epochs, batch=batch, lr=lr, wd=wd, seed=seed)
    params2 = None
    if ensemble:
        net2 = Mlp(init_params(seed + 1000))
        net2.train(Xs, Ys, epochs=epochs, batch=batch, lr=lr, wd=wd, seed=seed + 1000)
        params2 = net2.get_params()
        net2.close()
    model = ClosureModel(net.get_params(), *st, params2=params2)
    err = None
    if nh > 0:
        err = heldout_error(net, model, X[perm[:nh]], Y[perm[:nh]])
    net.close()
    return model, hist, err


def heldout_error(net, model, X, Y):
    """Median and 95th percentile relative errors of kQ and kT on (X, Y)."""
    Z = np.zeros_like(X)
    Z[:, :N_FEAT] = ((X[:, :N_FEAT] - model.fmu) / model.fsd).astype(np.float32)
    out = net.forward(Z).astype(np.float64) * model.ysd + model.ymu
    Yd = Y.astype(np.float64)
    # log kQ = y1, log kT + log(s^2 A_int) = y1 - y2
    lg = np.column_stack([out[:, 0], out[:, 0] - out[:, 1]])
    lt = np.column_stack([Yd[:, 0], Yd[:, 0] - Yd[:, 1]])
    rel = np.abs(np.expm1(lg - lt))
    return {"kQ_p50": float(np.median(rel[:, 0])), "kQ_p95": float(np.percentile(rel[:, 0], 95)),
            "kT_p50": float(np.median(rel[:, 1])), "kT_p95": float(np.percentile(rel[:, 1], 95))}


# ---- runs ----------------------------------------------------------------------
def run_plain(p, times, max_steps=1000000):
    """Plain FP64 run; at each time of `times` the total water content and
    the macro heads.  Returns (records, wall seconds, steps, G evaluations)."""
    ctx = P.Context(p)
    lib = ctx.lib
    check(lib.tsr_exprem_load(ctx.h, ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    t = C.c_double(0.0)
    tspan = np.array([0.0])
    u = np.empty(p.N)
    rec = []
    check(lib.tsr_sync(ctx.h), "sync")
    w0 = time.perf_counter()
    wall = 0.0
    for tk in times:
        while t.value < tk and st.NumSteps < max_steps:
            check(lib.tsr_exprem_advance(ctx.h, tk, ptr(tspan), None, C.byref(p.options), C.byref(st),
                                         C.byref(t)), "advance")
        check(lib.tsr_sync(ctx.h), "sync")
        wall += time.perf_counter() - w0
        check(lib.tsr_exprem_store(ctx.h, ptr(u)), "store")
        rec.append((t.value, ctx.water(u), u[:p.Mn].copy()))
        w0 = time.perf_counter()
    ctx.close()
    return rec, wall, st.NumSteps, st.FuncEvals


def run_closure(p, model, times, thr=1e-3, qfloor_rel=1e-3, auto_fallback=True, max_steps=1000000,
                params=None, t_switch=0.0, thr_ens=None, params2=None):
    """The same run with the learned closure: the plain method up to
    t_switch (0: none), then every cell learned; flagged cells fall back to
    their micro meshes.  thr_ens (with a second network, params2 or the
    model's): the two-network ensemble and its disagreement indicator.
    Returns (records, wall seconds, steps, G evaluations, fallback fraction
    per record time); the wall time includes the plain start."""
    p.set_learned(np.zeros(p.Ne, dtype=np.int32))      # full layout, closure enabled
    ctx = P.Context(p)
    lib = ctx.lib
    net = Mlp(model.params if params is None else params)
    net2 = None
    if thr_ens is not None:
        p2 = model.params2 if params2 is None else params2
        if p2 is None:
            raise ValueError("the ensemble indicator needs a second network")
        net2 = Mlp(p2)
    check(lib.tsr_exprem_load(ctx.h, ptr(p.u0), 0.0), "load")
    st = capi.ExpremStats()
    t = C.c_double(0.0)
    tspan = np.array([0.0])
    check(lib.tsr_sync(ctx.h), "sync")
    w_start = time.perf_counter()
    while t.value < t_switch and st.NumSteps < max_steps:
        check(lib.tsr_exprem_advance(ctx.h, t_switch, ptr(tspan), None, C.byref(p.options), C.byref(st),
                                     C.byref(t)), "advance")
    check(lib.tsr_sync(ctx.h), "sync")
    wall0 = time.perf_counter() - w_start
    # flux floor: a fraction of the largest plain exchange inflow at t = 0
    summ = np.empty(5 * p.Ne)
    check(lib.tsr_cell_summary(ctx.h, None, ptr(summ)), "summary")
    q0 = float(np.max(np.abs(summ.reshape(-1, 5)[:, 3])))
    ones = np.ones(p.Ne, dtype=np.int32)
    check(lib.tsr_closure_set_learned(ctx.h, ones.ctypes.data_as(capi.ip)), "set_learned")
    norm, zr = model.norm(), model.zrange()      # alive for the duration of the calls
    check(lib.tsr_closure_attach(ctx.h, net.h, ptr(norm), zr.ctypes.data_as(capi.fp),
                                 thr, qfloor_rel * q0, int(auto_fallback)), "attach")
    if net2 is not None:
        check(lib.tsr_closure_attach_ensemble(ctx.h, net2.h, thr_ens), "attach ensemble")
    # inputs of the network at t = 0 against the accepted range (diagnostic)
    S0 = summ.reshape(-1, 5)
    f0 = features(S0[:, 0], np.full((p.Ne, 3), np.nan), [0.0, -1e30, -1e30, -1e30], S0[:, 1], S0[:, 4])
    z0 = (f0 - model.fmu) / model.fsd
    ood0 = [float(np.mean((z0[:, i] < model.zlo[i]) | (z0[:, i] > model.zhi[i]))) for i in range(N_FEAT)]
    nf = C.c_int()
    rec, frac = [], []
    learned = np.empty(p.Ne, dtype=np.int32)
    check(lib.tsr_sync(ctx.h), "sync")
    w0 = time.perf_counter()
    wall = wall0
    nfl = []
    for tk in times:
        while t.value < tk and st.NumSteps < max_steps:
            check(lib.tsr_closure_advance(ctx.h, tk, ptr(tspan), None, C.byref(p.options), C.byref(st),
                                          C.byref(t), C.byref(nf)), "closure_advance")
            nfl.append(nf.value)
        check(lib.tsr_sync(ctx.h), "sync")
        wall += time.perf_counter() - w0
        n = lib.tsr_num_unknowns(ctx.h)
        u = np.empty(n)
        check(lib.tsr_exprem_store(ctx.h, ptr(u)), "store")
        w = C.c_double()
        check(lib.tsr_water_content(ctx.h, ptr(u), C.byref(w)), "water")
        check(lib.tsr_closure_read(ctx.h, learned.ctypes.data_as(capi.ip), None, None), "read")
        rec.append((t.value, w.value, u[:p.Mn].copy()))
        frac.append(1.0 - learned.mean())
        w0 = time.perf_counter()
    ctx.close()
    net.close()
    if net2 is not None:
        net2.close()
    run_closure.ood_t0 = ood0
    run_closure.flagged_per_step = nfl
    return rec, wall, st.NumSteps, st.FuncEvals, frac


def training_set(time_limit=45.0, skip=1, log=print, t_stop=None, n_macro=101):
    """Training data from plain runs of the CPU-runnable configuration (two
    initial heads drawn from seeds 1001-1002) and of the GPU-scale plain
    configuration at 101 x 101 macro nodes (inclusion sizes and initial
    noise from seeds 1001-1002; n_macro), each run for at most time_limit
    seconds and to at most t_stop days, from step `skip` on (the early steps carry the fast decay of the initial
    noise, whose head rates a closure run meets at its start too).  Returns
    (X, Y, description)."""
    X, Y, desc = [], [], []
    for seed in (1001, 1002):
        q = P.config1()
        h0 = float(np.random.default_rng(seed).uniform(-8.0, -2.0))
        q.u0 = q.initial_state(h0)
        logs = log_plain_run(q, time_limit=time_limit)
        x, y = samples(q, logs, skip=skip)
        X.append(x)
        Y.append(y)
        desc.append("21x21/11x11 h0=%.2f: %d steps to t=%.3g d, %d samples" % (h0, len(logs) - 1, logs[-1][0], len(x)))
        log(desc[-1])
    for seed in (1001, 1002):
        q = P.config2(n_macro=n_macro, seed=seed, eval_seed=seed + 1000)
        logs = log_plain_run(q, cell_stride=2, time_limit=time_limit, t_stop=t_stop)
        x, y = samples(q, logs, cell_stride=2, skip=skip)
        X.append(x)
        Y.append(y)
        desc.append("%dx%d/21x21 seed %d: %d steps to t=%.3g d, %d samples (every 2nd cell)"
                    % (n_macro, n_macro, seed, len(logs) - 1, logs[-1][0], len(x)))
        log(desc[-1])
    return np.concatenate(X), np.concatenate(Y), desc
