"""Learned moment surrogate and the surrogate-assisted Method-of-Moments fit.

The reference has no surrogate: every Robbins-Monro iteration of R/mom.R
simulates. Here a multilayer perceptron learns, per period, the map from the
period's parameters (and a summary of its observed start wave) to the expected
period statistics, from moments the GPU simulator itself generates. The
network is trained and evaluated by the kernels of csrc/mlp.cu (bfloat16
tensor-core products, float32 accumulation, Adam) through the C ABI
cusna_mlp_*; device buffers are torch tensors (allocation only).

Surrogate-assisted fit (`mom_run_surrogate`), a sequential design in stages
that share one budget of training pairs (default 65,536):
  1. training data: thetas drawn around the stage's centre -- the first
     stage theta ~ centre + N(0, 0.5^2 I), later stages in standard-error
     units of the previous stage (theta + c L z, L L^T the sandwich
     covariance) -- every period simulated once per draw in one batched
     launch (the simulator honours per-chain theta);
  2. training: a float64 quadratic response surface per period (host) plus
     the network on its residual (Adam on the GPU), the network's term gated
     per output by its held-out accuracy;
  3. phases 1-2 of R/mom.R:215-248 run on the surrogate: its mean replaces the
     simulated mean and its Jacobian replaces the score-function derivative,
     inside the stage's trust region (the box of its training thetas);
  4. between stages a plain pilot simulation at the estimate corrects it (a
     Newton step with the surrogate's Jacobian) and measures the covariance
     that scales the next stage's design (drawn within the previous stage's
     trust region widened by its width on each side); when the pilots' steps
     do not fall below a standard error, the surrogate is not trusted and
     plain simulation takes over (the Robbins-Monro phases of R/mom.R from
     the fit's start);
  5. phase 3 (R/mom.R:250-258) simulates as in the plain fit and judges the
     surrogate: its error is |simulated mean - surrogate mean| / simulated SD
     per statistic. When that error, or a convergence t-ratio, reaches the
     bound (0.1), plain simulation takes over: a Newton step with the phase-3
     derivative and another phase 3, until the t-ratios are within the bound,
     and the plain Robbins-Monro phases when a few such steps do not get there
     (from the last point when it is near the targets, else from the start).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import mom
from .abi import adam_hyper_bytes, check, load_library

N_IN = 16          # surrogate input width: period parameters + start-wave features
HIDDEN = 256


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the moment surrogate runs on the GPU only (no CPU path)")
    return torch


class MlpSurrogate:
    """n_in -> hidden -> hidden -> n_out GELU network on the GPU, with input and
    output standardisation kept on the host and a polynomial shortcut:

        y_std = phi(x_std) C_g + r_sd * net(x_std)

    phi is the degree-1 or degree-2 monomial basis of the varying inputs (the
    first n_in - n_group; the last n_group inputs are constant within a group,
    here a period's start-wave features) and C_g the float64 least-squares
    coefficients of group g, fitted on the host. The network learns the
    standardised residual: what the response surface leaves. Without it
    (degree=0) the shortcut is zero and r_sd = 1."""

    def __init__(self, n_in: int = N_IN, n_out: int = 8, hidden: int = HIDDEN, seed: int = 0):
        torch = _torch()
        self.lib = load_library()
        self.n_in, self.n_out, self.hidden = int(n_in), int(n_out), int(hidden)
        self.dev = torch.device("cuda", torch.cuda.current_device())
        npar = int(self.lib.cusna_mlp_param_count(self.n_in, self.hidden, self.n_out))
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.params = torch.empty(npar, **f32)
        self.grad = torch.zeros(npar, **f32)
        self.adam_m = torch.zeros(npar, **f32)
        self.adam_v = torch.zeros(npar, **f32)
        self.step = 0
        self._work = None
        self._work_bytes = 0
        check(self.lib.cusna_mlp_init(self.params.data_ptr(), self.n_in, self.hidden, self.n_out,
                                      C.c_uint64(int(seed)), self._stream()),
              "cusna_mlp_init", self.lib)
        self.x_mu = np.zeros(self.n_in)
        self.x_sd = np.ones(self.n_in)
        self.y_mu = np.zeros(self.n_out)
        self.y_sd = np.ones(self.n_out)
        self.degree = 0           # shortcut degree (0: none)
        self.Cg = []              # per-group shortcut coefficients (basis x n_out)
        self.C = None             # pooled coefficients (rows of unseen groups)
        self.groups = None        # distinct trailing-feature vectors
        self.n_group = 0
        self.r_sd = np.ones(self.n_out)
        self.alpha = np.ones(self.n_out)  # per-output gate of the network term
        self.use_graph = True             # replay each training epoch from a CUDA graph
        self.history: list = []

    def _stream(self):
        return self._torch.cuda.current_stream(self.dev).cuda_stream

    @property
    def _torch(self):
        import torch
        return torch

    def _workspace(self, batch: int):
        need = int(self.lib.cusna_mlp_workspace_bytes(self.n_in, self.hidden, self.n_out, int(batch)))
        if need > self._work_bytes:
            self._work = self._torch.empty(need, dtype=self._torch.uint8, device=self.dev)
            self._work_bytes = need
        return self._work.data_ptr(), self._work_bytes

    def set_scaling(self, X, Y):
        X, Y = np.asarray(X, dtype=np.float64), np.asarray(Y, dtype=np.float64)
        self.x_mu, self.y_mu = X.mean(axis=0), Y.mean(axis=0)
        self.x_sd = np.maximum(X.std(axis=0), 1e-6)
        self.y_sd = np.maximum(Y.std(axis=0), 1e-6)

    def _dev(self, a):
        return self._torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(self.dev)

    def _group_of(self, X):
        """Group index of each row (rows grouped by their last n_group
        inputs); -1 for a feature vector not seen in training."""
        if not self.n_group or self.groups is None:
            return np.zeros(X.shape[0], dtype=int)
        g = np.full(X.shape[0], -1)
        F = X[:, self.n_in - self.n_group:]
        for i, key in enumerate(self.groups):
            g[np.all(F == key[None, :], axis=1)] = i
        return g

    def _basis(self, xs):
        """Monomials of the varying standardised inputs up to self.degree:
        [x_1..x_v, x_i x_j (i <= j) if degree 2, 1]."""
        v = self.n_in - self.n_group
        z = xs[:, :v]
        cols = [z]
        if self.degree >= 2:
            iu, ju = np.triu_indices(v)
            cols.append(z[:, iu] * z[:, ju])
        cols.append(np.ones((xs.shape[0], 1)))
        return np.hstack(cols)

    def _basis_jac(self, xs, n_wrt):
        """d basis / d xs[:, :n_wrt], (B, n_basis, n_wrt)."""
        v = self.n_in - self.n_group
        B = xs.shape[0]
        z = xs[:, :v]
        parts = [np.broadcast_to(np.eye(v)[:, :n_wrt], (B, v, n_wrt))]
        if self.degree >= 2:
            iu, ju = np.triu_indices(v)
            Jq = np.zeros((B, len(iu), n_wrt))
            for c, (i, j) in enumerate(zip(iu, ju)):
                if i < n_wrt:
                    Jq[:, c, i] += z[:, j]
                if j < n_wrt:
                    Jq[:, c, j] += z[:, i]
            parts.append(Jq)
        parts.append(np.zeros((B, 1, n_wrt)))
        return np.concatenate(parts, axis=1)

    def _coef_rows(self, X):
        g = self._group_of(X)
        return [self.Cg[i] if i >= 0 else self.C for i in g]

    def _shortcut(self, xs, X):
        if not self.degree:
            return np.zeros((xs.shape[0], self.n_out))
        Phi = self._basis(xs)
        return np.einsum("bk,bko->bo", Phi, np.stack(self._coef_rows(X)))

    def _shortcut_jac(self, xs, X, n_wrt):
        if not self.degree:
            return np.zeros((xs.shape[0], self.n_out, n_wrt))
        Jb = self._basis_jac(xs, n_wrt)
        return np.einsum("bkw,bko->bow", Jb, np.stack(self._coef_rows(X)))

    def fit(self, X, Y, epochs: int = 40, batch: int = 1024, lr: float = 2e-3,
            lr_final: float = 5e-5, val_frac: float = 0.05, seed: int = 0,
            degree: int = 2, n_group: int = 0) -> dict:
        """Adam on the standardised pairs (residuals of the polynomial
        shortcut of the given degree) with a cosine learning-rate decay,
        keeping the parameters of the epoch with the lowest validation loss;
        returns the per-epoch training and validation losses (mean squared
        error of the standardised residual). n_group > 0 fits one shortcut per
        distinct value of the last n_group inputs."""
        torch = self._torch
        X, Y = np.asarray(X, dtype=np.float64), np.asarray(Y, dtype=np.float64)
        N = X.shape[0]
        rng = np.random.Generator(np.random.PCG64(seed))
        order = rng.permutation(N)
        n_val = int(round(val_frac * N))
        val, tr = order[:n_val], order[n_val:]
        self.set_scaling(X[tr], Y[tr])
        xs, ys = (X - self.x_mu) / self.x_sd, (Y - self.y_mu) / self.y_sd
        self.degree, self.n_group = int(degree), int(n_group)
        if self.degree:
            Phi = self._basis(xs)

            def lsq(rows):
                return np.linalg.lstsq(Phi[rows], ys[rows], rcond=None)[0]
            self.C = lsq(tr)
            self.groups = (np.unique(X[:, self.n_in - self.n_group:], axis=0)
                           if self.n_group else None)
            g = self._group_of(X)
            ng = len(self.groups) if self.n_group else 1
            self.Cg = [lsq(tr[g[tr] == i]) if np.sum(g[tr] == i) > 4 * Phi.shape[1] else self.C
                       for i in range(ng)]
            R = ys - self._shortcut(xs, X)
            self.r_sd = np.maximum(R[tr].std(axis=0), 1e-12)
            ys = R / self.r_sd
        Xs = self._dev(xs)
        Ys = self._dev(ys)
        batch = int(batch) - int(batch) % 16
        steps = len(tr) // batch
        if steps < 1:
            raise ValueError("fewer training rows than one batch")
        wp, wb = self._workspace(batch)
        losses = torch.zeros(steps, dtype=torch.float32, device=self.dev)
        val_idx = torch.from_numpy(val.astype(np.int64)).to(self.dev)
        st = self._stream()
        t0 = time.perf_counter()
        best, best_params = np.inf, None
        # one epoch = `steps` Adam steps replayed from a CUDA graph: the
        # permutation buffer and the learning rate (device-side) change
        # between replays, the arguments do not
        perm = torch.empty(len(tr), dtype=torch.int32, device=self.dev)
        hyper = torch.from_numpy(adam_hyper_bytes(self.step, lr)).to(self.dev)
        for ep in range(epochs):
            perm.copy_(torch.from_numpy(rng.permutation(tr).astype(np.int32)))
            lr_ep = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * ep / max(epochs, 1)))
            hyper[4:8].copy_(torch.from_numpy(np.array([lr_ep], dtype=np.float32).view(np.uint8)))
            st_ = self.lib.cusna_mlp_train_steps(
                self.params.data_ptr(), self.grad.data_ptr(), self.adam_m.data_ptr(),
                self.adam_v.data_ptr(), Xs.data_ptr(), Ys.data_ptr(), perm.data_ptr(), batch,
                steps, hyper.data_ptr(), losses.data_ptr(), wp, wb, self.n_in, self.hidden,
                self.n_out, 1 if self.use_graph else 0, st)
            check(st_, "cusna_mlp_train_steps", self.lib)
            self.step += steps
            rec = dict(epoch=ep, lr=lr_ep, train=float(losses.mean().item()))
            if n_val:
                rec["val"] = self._std_mse(Xs[val_idx], Ys[val_idx])
                if rec["val"] < best:
                    best = rec["val"]
                    best_params = self.params.clone()
            self.history.append(rec)
        if best_params is not None:
            self.params.copy_(best_params)
        if n_val:
            # per-output gate: least-squares shrinkage of the network's residual
            # prediction on the held-out rows, in [0, 1] (0 when the network
            # does not predict the residual better than zero does)
            net = self._forward_std(Xs[val_idx]).double().cpu().numpy()
            Rv = ys[val]
            self.alpha = np.clip((net * Rv).sum(axis=0) / np.maximum((net * net).sum(axis=0), 1e-30),
                                 0.0, 1.0)
            # what the network adds: held-out mean squared error per output, in
            # units of the response surface's residual SD, of the response
            # surface alone (the residual itself) and with the gated network
            val_surface = (Rv * Rv).mean(axis=0)
            val_net = ((Rv - self.alpha * net) ** 2).mean(axis=0)
        else:
            val_surface = val_net = None
        torch.cuda.synchronize(self.dev)
        return dict(history=self.history, seconds=time.perf_counter() - t0, steps=steps * epochs,
                    batch=batch, n_train=len(tr), n_val=n_val, best_val=best,
                    val_surface=val_surface, val_net=val_net)

    def _std_mse(self, Xs, Ys) -> float:
        y = self._forward_std(Xs)
        return float(((y - Ys) ** 2).mean().item())

    def _forward_std(self, Xs):
        torch = self._torch
        B = Xs.shape[0]
        y = torch.empty((B, self.n_out), dtype=torch.float32, device=self.dev)
        wp, wb = self._workspace(B)
        check(self.lib.cusna_mlp_forward(self.params.data_ptr(), Xs.contiguous().data_ptr(), B,
                                         y.data_ptr(), wp, wb, self.n_in, self.hidden,
                                         self.n_out, self._stream()),
              "cusna_mlp_forward", self.lib)
        return y

    def predict(self, X) -> np.ndarray:
        """Surrogate outputs in the original units, (B, n_out)."""
        X = np.atleast_2d(np.asarray(X, dtype=np.float64))
        xs = (X - self.x_mu) / self.x_sd
        y = self._forward_std(self._dev(xs)).double().cpu().numpy()
        return (self._shortcut(xs, X) + self.gain * y) * self.y_sd + self.y_mu

    @property
    def gain(self):
        return self.r_sd * self.alpha

    def predict_with_jacobian(self, X, n_wrt: int):
        """(outputs (B, n_out), Jacobian (B, n_out, n_wrt)) in original units
        with respect to the first n_wrt inputs."""
        torch = self._torch
        X = np.atleast_2d(np.asarray(X, dtype=np.float64))
        xs = (X - self.x_mu) / self.x_sd
        Xs = self._dev(xs)
        B = Xs.shape[0]
        y = torch.empty((B, self.n_out), dtype=torch.float32, device=self.dev)
        J = torch.empty((B, self.n_out, n_wrt), dtype=torch.float32, device=self.dev)
        wp, wb = self._workspace(B)
        check(self.lib.cusna_mlp_jacobian(self.params.data_ptr(), Xs.data_ptr(), B, int(n_wrt),
                                          y.data_ptr(), J.data_ptr(), wp, wb, self.n_in,
                                          self.hidden, self.n_out, self._stream()),
              "cusna_mlp_jacobian", self.lib)
        y = (self._shortcut(xs, X) + self.gain * y.double().cpu().numpy()) * self.y_sd + self.y_mu
        Js = self._shortcut_jac(xs, X, n_wrt) + self.gain[None, :, None] * J.double().cpu().numpy()
        J = Js * self.y_sd[None, :, None] / self.x_sd[None, None, :n_wrt]
        return y, J

    def params_host(self) -> np.ndarray:
        return self.params.double().cpu().numpy()

    def load_params(self, p) -> None:
        self.params.copy_(self._torch.from_numpy(np.asarray(p, dtype=np.float32)))


# ---- the per-period decomposition of the estimator --------------------------
def period_blocks(est: mom.Estimator) -> list:
    """Indices of the parameter vector (equally of the statistic vector) that
    period q's simulation reads and fills: its rate(s) and every shared
    evaluation/behaviour parameter (the layouts of R/mom.R:131-138)."""
    P, k, p = est.P, est.k, est.p
    if est.coevol:
        shared = list(range(2 * P, p))
        return [np.array([q, P + q] + shared) for q in range(P)]
    if est.conditional:
        return [np.arange(k) for _ in range(P)]
    return [np.array([q] + list(range(P, p))) for q in range(P)]


def period_features(est: mom.Estimator, engine, n_feat: int) -> np.ndarray:
    """Summary of each period's observed start wave, (P, n_feat): the k model
    statistics of the start network, then its mean outdegree, its observed
    distance to the next wave and the actor count, cut or zero-padded to
    n_feat."""
    out = np.zeros((est.P, n_feat))
    for q in range(est.P):
        inp = est.per[q]["inp"]
        a = np.asarray(inp.x0)
        od0 = a.sum(axis=1).astype(np.int32)
        id0 = a.sum(axis=0).astype(np.int32)
        s = engine.network_stats(a, est.n, est.k, inp.type_ids, inp.p1, inp.p2, inp.vmat,
                                 inp.vmiss, inp.dyn_flags, inp.vb, od0, id0, inp.wtab,
                                 est.symflag)
        f = list(np.ravel(s)) + [a.sum() / max(est.n, 1), est.dists[q], float(est.n)]
        f = f[:n_feat]
        out[q, :len(f)] = f
    return out



@dataclass
class Stage:
    """One round of the sequential training design: `frac` of the training
    pairs, drawn around the current estimate either isotropically
    (theta + spread * N(0, I)) or in standard-error units (theta + spread * L z
    with L L^T the sandwich covariance of the previous stage's surrogate)."""
    frac: float
    design: str          # "iso" or "se"
    spread: float
    epochs: int = 40


DEFAULT_STAGES = (Stage(0.25, "iso", 0.5, 60), Stage(0.75, "se", 2.0, 30))


@dataclass
class SurrogateControl:
    """Settings of the surrogate-assisted fit."""
    n_pairs: int = 65536          # (theta, period moments) training pairs over all stages
    stages: tuple = DEFAULT_STAGES
    hidden: int = HIDDEN
    batch: int = 1024
    lr: float = 2e-3
    bound: float = 0.1            # judge bound on surrogate error and t-ratios
    max_takeovers: int = 3        # plain Newton corrections after the judge fails
    pilot: int = 1000             # chains of each plain pilot between stages
    max_pilots: int = 4           # pilots between two stages at most
    pilot_tol: float = 1.0        # stop piloting once a step is below this many SEs
    seed: int = 4321
    network: bool = True          # False: the response surface alone (no network term)


@dataclass
class SurrogateFit:
    fit: mom.MomFit
    judge: list = field(default_factory=list)     # per phase-3 round: errors, t-ratios
    takeovers: int = 0
    stages: list = field(default_factory=list)    # per stage: design, estimate, training
    theta_surrogate: np.ndarray | None = None
    n_period_sims: int = 0
    fallback: str | None = None     # why plain simulation took over before phase 3


class PanelSurrogate:
    """The estimator's expected statistics and Jacobian from a per-period
    network: E[s](theta) = sum over periods of g([theta[block_q], f_q])
    placed at block_q."""

    def __init__(self, est: mom.Estimator, net: MlpSurrogate, feats: np.ndarray):
        self.est, self.net, self.feats = est, net, feats
        self.blocks = period_blocks(est)

    def inputs(self, theta) -> np.ndarray:
        rows = []
        for q, b in enumerate(self.blocks):
            rows.append(np.concatenate([np.asarray(theta)[b], self.feats[q]]))
        return np.array(rows)

    def mean_and_jacobian(self, theta):
        d = len(self.blocks[0])
        y, J = self.net.predict_with_jacobian(self.inputs(theta), d)
        p = self.est.p
        mean, D = np.zeros(p), np.zeros((p, p))
        for q, b in enumerate(self.blocks):
            mean[b] += y[q]
            D[np.ix_(b, b)] += J[q]
        return mean, D

    def mean(self, theta):
        y = self.net.predict(self.inputs(theta))
        mean = np.zeros(self.est.p)
        for q, b in enumerate(self.blocks):
            mean[b] += y[q]
        return mean


def draw_thetas(est: mom.Estimator, centre, n_theta, rng, design, spread, chol=None,
                limit=None):
    """Training parameter vectors: centre + spread * z (design "iso") or
    centre + spread * chol z (design "se"); rates are kept positive, and every
    coordinate within `limit` (lo, hi) when given."""
    p = est.p
    z = rng.standard_normal((n_theta, p))
    centre = np.asarray(centre, dtype=np.float64)
    theta = centre[None, :] + spread * (z if design == "iso" else z @ chol.T)
    if limit is not None:
        theta = np.clip(theta, limit[0], limit[1])
    n_rates = 0 if est.conditional else (2 * est.P if est.coevol else est.P)
    if n_rates:
        theta[:, :n_rates] = np.maximum(theta[:, :n_rates], 0.05 * np.abs(centre[:n_rates]) + 1e-3)
    return theta


def training_pairs(est: mom.Estimator, theta, rng, engine, feats):
    """Simulate every period once for each row of `theta` (all periods in one
    batch launch) and return the per-period (input, statistics) pairs, period
    after period: (P * rows, N_IN) and (P * rows, d)."""
    blocks = period_blocks(est)
    n_theta = theta.shape[0]
    s = mom.mom_simulate(est, theta[0], n_theta, rng, engine, theta_rows=theta, scores=False)
    X, Y = [], []
    for q, (sp, _) in enumerate(s.pieces):
        b = blocks[q]
        X.append(np.hstack([theta[:, b], np.repeat(feats[q][None, :], n_theta, axis=0)]))
        Y.append(sp[:, b])
    return np.vstack(X), np.vstack(Y)


def pilot_correction(est: mom.Estimator, sur: PanelSurrogate, theta, M, rng, engine, box):
    """Plain simulation between stages: M chains at theta give the simulated
    mean, the covariance S of the summed statistics and the score-function
    derivative D (R/mom.R:173-182, as plain phase 1 estimates it). Returns the
    Newton point theta - D^-1 (mean - targets) (guarded, and kept within the
    surrogate's trust region `box` widened by its own width on each side),
    the Cholesky factor of D^-1 S D^-T (the sandwich covariance, one
    simulation's) that scales the next stage's design (its diagonal when not
    positive definite), the simulated mean and the statistics' SDs."""
    s = mom.mom_simulate(est, theta, M, rng, engine)
    mean = s.stats.mean(axis=0)
    S = np.atleast_2d(np.cov(s.stats, rowvar=False))
    Di = mom.safe_solve(mom.mom_derivative(s.pieces))
    lo, hi = box
    nxt = np.clip(theta - mom.guard_step(est, theta, Di @ (mean - est.targets)),
                  lo - (hi - lo), hi + (hi - lo))
    cov = Di @ S @ Di.T
    cov = 0.5 * (cov + cov.T)
    try:
        chol = np.linalg.cholesky(cov)
    except np.linalg.LinAlgError:
        chol = np.diag(np.sqrt(np.abs(np.diag(cov))))
    return nxt, chol, mean, np.sqrt(np.maximum(np.diag(S), 1e-300))


def design_box(th, q=0.005):
    """Per-coordinate trust region of a surrogate: the q and 1-q quantiles of
    its training thetas."""
    return np.quantile(th, q, axis=0), np.quantile(th, 1 - q, axis=0)


def _rm_on_surrogate(est, sur: PanelSurrogate, theta, ctl, box):
    """Phases 1-2 of R/mom.R:215-248 with the surrogate's mean in place of the
    simulated mean and its Jacobian in place of the score-function derivative.
    Every iterate is clipped to the surrogate's trust region `box` (lo, hi):
    the surrogate is never evaluated where it saw no training data, so an
    extrapolation cannot drive a rate (and the next simulation's length)
    without bound."""
    lo, hi = box

    def step(th, delta):
        return np.clip(th - mom.guard_step(est, th, delta), lo, hi)
    theta = np.clip(theta, lo, hi)
    mean, Dm = sur.mean_and_jacobian(theta)
    dinv = mom.mom_dinv(Dm, ctl["diagonalize"])
    theta = step(theta, 0.5 * ctl["firstg"] * (dinv @ (mean - est.targets)))
    n2 = list(ctl["n2"])
    for sub in range(ctl["nsub"]):
        gain = ctl["firstg"] * (0.5 ** sub)
        _, Dm = sur.mean_and_jacobian(theta)
        dinv = mom.mom_dinv(Dm, ctl["diagonalize"])
        thav = np.zeros(est.p)
        for _ in range(int(n2[sub])):
            theta = step(theta, gain * (dinv @ (sur.mean(theta) - est.targets)))
            thav += theta
        theta = thav / n2[sub]
    return theta


def mom_run_surrogate(est: mom.Estimator, centre, scontrol: SurrogateControl | None = None,
                      engine=None, verbose=False) -> SurrogateFit:
    """Surrogate-assisted fit (module docstring). `centre` is the design centre
    of the first stage's training thetas (a prior estimate; also where the
    surrogate's Robbins-Monro starts)."""
    sc = scontrol or SurrogateControl()
    engine = engine or mom.GpuEngine()
    ctl = est.control
    t0 = time.perf_counter()
    times = dict(simulate_training=0.0, train=0.0, surrogate_rm=0.0)
    rng = np.random.Generator(np.random.PCG64(int(sc.seed)))
    theta = np.asarray(centre, dtype=np.float64).copy()
    d = len(period_blocks(est)[0])
    n_feat = N_IN - d
    if n_feat < 0:
        raise ValueError(f"{d} parameters per period exceed the surrogate input width {N_IN}")
    feats = period_features(est, engine, n_feat)
    stages, sur, chol, n_theta_total, n_pilot = [], None, None, 0, 0
    limit, fallback = None, None
    for i, stg in enumerate(sc.stages):
        n_theta = max(16, -(-int(round(stg.frac * sc.n_pairs)) // est.P))
        design = stg.design if (stg.design == "iso" or chol is not None) else "iso"
        ta = time.perf_counter()
        th = draw_thetas(est, theta, n_theta, rng, design, stg.spread, chol, limit)
        X, Y = training_pairs(est, th, rng, engine, feats)
        times["simulate_training"] += time.perf_counter() - ta
        n_theta_total += n_theta
        ta = time.perf_counter()
        net = MlpSurrogate(N_IN, d, sc.hidden, seed=sc.seed + i)
        # without the network the fit trains no epochs: the untrained network
        # predicts zero, so its gated term is zero and the surface stands alone
        info = net.fit(X, Y, epochs=stg.epochs if sc.network else 0, batch=sc.batch, lr=sc.lr,
                       seed=sc.seed + i, n_group=n_feat)
        if not sc.network:
            net.alpha = np.zeros(net.n_out)
        times["train"] += time.perf_counter() - ta
        sur = PanelSurrogate(est, net, feats)
        ta = time.perf_counter()
        box = design_box(th)
        theta = _rm_on_surrogate(est, sur, theta.copy(), ctl, box)
        times["surrogate_rm"] += time.perf_counter() - ta
        rec = dict(design=design, spread=stg.spread, n_theta=n_theta, theta=theta.copy(),
                   train_seconds=info["seconds"], val=info.get("best_val"),
                   gate=net.alpha.copy(), val_surface=info.get("val_surface"),
                   val_net=info.get("val_net"))
        if i + 1 < len(sc.stages):
            # plain pilots with the surrogate's Jacobian (quasi-Newton) until
            # the step is below pilot_tol standard errors in every coordinate
            ta = time.perf_counter()
            rec["pilot_steps"] = []
            step_se = np.inf
            for _ in range(sc.max_pilots):
                prev = theta
                theta, chol, pmean, psd = pilot_correction(est, sur, theta, sc.pilot, rng, engine, box)
                n_pilot += sc.pilot
                step_se = float(np.max(np.abs(theta - prev) / np.sqrt(np.diag(chol @ chol.T)).clip(1e-300)))
                rec["pilot_steps"].append(step_se)
                if "pilot_error" not in rec:
                    rec["pilot_error"] = np.abs(pmean - sur.mean(prev)) / psd
                if step_se < sc.pilot_tol:
                    break
            times["pilot"] = times.get("pilot", 0.0) + time.perf_counter() - ta
            rec["theta_corrected"] = theta.copy()
            # the next stage's draws stay inside this stage's trust region
            # widened by its own width on each side, as the pilots do
            limit = (box[0] - (box[1] - box[0]), box[1] + (box[1] - box[0]))
            if step_se >= sc.pilot_tol:
                # the surrogate's estimate did not hold up under the plain
                # pilots: the surrogate is not trusted further, and plain
                # simulation takes over (the Robbins-Monro phases of R/mom.R
                # from the last pilot's point)
                fallback = "pilot steps did not fall below pilot_tol standard errors"
        stages.append(rec)
        if verbose:
            print(f"[surrogate stage {i + 1}: {design} x{stg.spread}] theta =", np.round(rec["theta"], 4),
                  "corrected =", np.round(theta, 4))
        if fallback:
            break
    def plain_takeover(theta, judge, takeovers, n_before):
        # plain simulation takes over: the Robbins-Monro phases of R/mom.R
        # from theta (a fit that does not depend on the surrogate any more)
        ta = time.perf_counter()
        plain = mom.mom_run(est, theta0=theta, engine=engine, verbose=verbose)
        times["plain_takeover"] = time.perf_counter() - ta
        n_sims = n_before + plain.n_sims
        fit = mom.MomFit(plain.theta, plain.se, plain.tconv, plain.tconv_max, est.param_names,
                         est.targets, plain.sim_means, plain.D, plain.msf, est.conditional,
                         plain.rate_est, plain.rate_sd, int(n_sims), time.perf_counter() - t0,
                         "gpu+surrogate (plain takeover)", None, None, times)
        return SurrogateFit(fit, judge, takeovers + 1, stages, theta_sur, n_sims * est.P, fallback)

    theta_sur = theta.copy()
    start = np.asarray(centre, dtype=np.float64).copy()
    if fallback:
        # the pilots wandered: the plain phases start again from the fit's start
        return plain_takeover(start, [], 0, n_theta_total + n_pilot)
    ta = time.perf_counter()
    theta, p3, judge, takeovers = judge_and_take_over(est, sur, theta, engine, rng, ctl["n3"],
                                                      sc.bound, sc.max_takeovers, verbose)
    times["phase3"] = time.perf_counter() - ta
    if not judge[-1]["passed"]:
        # the judge's Newton steps did not reach the bound either: the plain
        # phases continue from the last phase-3 point when it is near the
        # targets (every |t-conv| below 3), else start again from the start
        fallback = "phase-3 Newton takeovers did not bring the t-ratios within the bound"
        near = bool(np.max(np.abs(judge[-1]["tconv"])) < 3.0)
        return plain_takeover(theta if near else start, judge, takeovers,
                              n_theta_total + n_pilot + ctl["n3"] * len(judge))
    s, Dm, msf, dev, tconv, tconv_max, se = p3
    rate_est = s.ntim.mean(axis=0) if est.conditional else None
    rate_sd = s.ntim.std(axis=0, ddof=1) if est.conditional else None
    n_sims = n_theta_total + n_pilot + ctl["n3"] * len(judge)
    fit = mom.MomFit(theta, se, tconv, tconv_max, est.param_names, est.targets,
                     s.stats.mean(axis=0), Dm, msf, est.conditional, rate_est, rate_sd,
                     int(n_sims), time.perf_counter() - t0, "gpu+surrogate", None, None, times)
    return SurrogateFit(fit, judge, takeovers, stages, theta_sur, n_sims * est.P)


def judge_and_take_over(est: mom.Estimator, sur, theta, engine, rng, n3, bound=0.1,
                        max_takeovers=3, verbose=False):
    """Phase 3 (R/mom.R:250-258) as the surrogate's judge. The surrogate's
    error at theta is |simulated mean - sur.mean(theta)| / simulated SD per
    statistic; it passes when that error and every convergence t-ratio are
    below `bound`. Otherwise plain simulation takes over: a guarded Newton
    step with the phase-3 derivative and another phase 3, until the t-ratios
    are below the bound or max_takeovers steps were taken. Returns (theta,
    the last phase-3 tuple, per-round records, takeovers)."""
    judge, takeovers = [], 0
    while True:
        p3 = mom.phase3(est, theta, engine, rng, n3)
        s, Dm, msf, dev, tconv, _, _ = p3
        sd = np.sqrt(np.maximum(np.diag(msf), 1e-300))
        err = np.abs(s.stats.mean(axis=0) - sur.mean(theta)) / sd
        converged = bool(np.max(np.abs(tconv)) < bound)
        # the surrogate passes when its own error is within the bound at its
        # estimate; after a takeover only the t-ratios decide
        ok = converged and (takeovers > 0 or bool(np.max(err) < bound))
        judge.append(dict(theta=theta.copy(), error=err, tconv=tconv, passed=ok,
                          takeover=takeovers > 0))
        if verbose:
            print(f"[judge] max error {np.max(err):.4f} max |t| {np.max(np.abs(tconv)):.4f}")
        if ok or takeovers >= max_takeovers:
            return theta, p3, judge, takeovers
        takeovers += 1     # plain simulation takes over: Newton step with the phase-3 D
        theta = theta - mom.guard_step(est, theta, mom.safe_solve(Dm) @ dev)
