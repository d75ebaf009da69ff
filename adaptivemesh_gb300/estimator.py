"""The learned refinement / error estimator (include/amr_gb300.h, amr_estimator_*): a per-tile
BF16 3-D convolutional network, trained on the GPU by the library's own forward and backward
kernels, on targets the solver generates itself.

  Estimator            the network (create, forward, gradients, train_step, parameters)
  richardson_samples   features, targets and plain indicators from paired coarse / fine runs of one
                       configuration:
                       for each leaf of the coarse run, log10 of the Richardson estimate of its
                       truncation error after a short evolution, (|u_coarse - u_fine| * 2^p / (2^p - 1),
                       p = 4, over the conformal factor and the lapse), with the features of the
                       coarse state it started from
  train                Adam steps over a sample set
  captured_error       the share of the true error held by the k leaves a criterion ranks highest
  calibrate            least-squares line log10(error) ~ a + b log10(plain indicator): the plain
                       criterion expressed as an error estimate, for thresholds in error units
  train_default        the network of the binary-puncture configuration (16^3 tiles), trained on
                       seeded jittered configurations, with the held-out error of both estimates;
                       save / load_trained keep it in an .npz file
                       (python -m adaptivemesh_gb300.estimator --out FILE trains one)

No counterpart in the reference, whose refinement criterion is a gradient / curvature threshold
(SimpleWave.h:91-187).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import (F_ALPHA, F_CHI, ID_BRILL_LINDQUIST, MODE_GRAPH, SIM_BSSN_EVOLVE, SLICING_1PLUSLOG, VP, Config,
               Evolution, InitialData, check, load)
from .octree import Sim


class Estimator:
    def __init__(self, max_batch: int = 256, seed: int = 1):
        h = VP()
        check(load().amr_estimator_create(max_batch, seed, ctypes.byref(h)), "amr_estimator_create")
        self.h, self.max_batch = h, max_batch

    @staticmethod
    def param_count() -> int:
        return int(load().amr_estimator_param_count())

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        check(load().amr_estimator_get_params(self.h, p.ctypes.data), "amr_estimator_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(load().amr_estimator_set_params(self.h, p.ctypes.data), "amr_estimator_set_params")

    def forward(self, features):
        """Predicted log10 errors of the tiles (a device tensor [n][3][512] in, a device tensor out)."""
        import torch
        features = features.contiguous()
        out = torch.empty(features.shape[0], dtype=torch.float32, device=features.device)
        check(load().amr_estimator_forward(self.h, features.data_ptr(), features.shape[0], out.data_ptr()),
              "amr_estimator_forward")
        return out

    def gradients(self, features, targets):
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float()
        check(load().amr_estimator_gradients(self.h, features.contiguous().data_ptr(), targets.contiguous().data_ptr(),
                                             features.shape[0], g.ctypes.data, ctypes.byref(loss)),
              "amr_estimator_gradients")
        return g, loss.value

    def train_step(self, features, targets, lr: float = 1e-3) -> float:
        loss = ctypes.c_float()
        check(load().amr_estimator_train_step(self.h, features.contiguous().data_ptr(),
                                              targets.contiguous().data_ptr(), features.shape[0], lr,
                                              ctypes.byref(loss)), "amr_estimator_train_step")
        return loss.value

    def close(self) -> None:
        if self.h:
            load().amr_estimator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def binary_punctures(seed: int, separation: float = 6.0, mass: float = 0.5, jitter: float = 0.01):
    """Two equal-mass punctures on the x axis with seeded positional jitter."""
    rng = np.random.default_rng(seed)
    out = []
    for sgn in (-1.0, 1.0):
        pos = np.array([sgn * separation / 2, 0.0, 0.0]) + rng.uniform(-jitter, jitter, 3)
        out.append((mass, tuple(float(v) for v in pos)))
    return out


def refine_around(sim, points, depth: int, outer: float, margin: float = 1.25) -> None:
    """Refine every domain that contains or touches one of the points down to `depth`: a domain is
    refined when a point lies within `margin` half-edges of its centre along every axis (1.25: the
    domain and a quarter of its neighbours; larger margins refine shells of neighbours too)."""
    for d in range(depth):
        st = sim.state()
        used, pos, ch = st["used_slots"], st["positions"], st["children"]
        parents, offsets = [], []
        for s in range(used):
            p = int(pos[s])
            if p == 0xFFFFFFFF or (p >> 27) != d:
                continue
            # centre and half edge of slot s
            c = np.zeros(3)
            path = p & ((1 << 27) - 1)
            for i in range(d):
                for a in range(3):
                    c[a] += (0.25 if path & (1 << a) else -0.25) / (1 << i)
                path >>= 3
            c *= outer
            half = outer / 2 / (1 << d)
            if not any(np.all(np.abs(np.asarray(q) - c) <= half * margin) for q in points):
                continue
            for o in range(8):
                if ch[s * 8 + o] == -1:
                    parents.append(s)
                    offsets.append(o)
        if parents:
            sim.add_nodes(parents, offsets)


def build_sim(n: int, outer: float, punctures, depth: int, extra_levels: int = 0, slots: int = 4096,
              mode: int = MODE_GRAPH):
    """A BSSN evolution of Brill-Lindquist punctures on an octree refined around them to `depth`,
    every leaf then refined `extra_levels` more times (the fine member of a Richardson pair)."""
    sim = Sim(Config(n, 3, outer), SIM_BSSN_EVOLVE, slots=slots, mode=mode)
    refine_around(sim, [p for _, p in punctures], depth, outer)
    for _ in range(extra_levels):
        st = sim.state()
        used, pos, ch = st["used_slots"], st["positions"], st["children"]
        leaves = [s for s in range(used) if pos[s] != 0xFFFFFFFF and all(c == -1 for c in ch[8 * s:8 * s + 8])]
        sim.add_nodes([s for s in leaves for _ in range(8)], [o for _ in leaves for o in range(8)])
    sim.set_evolution(Evolution(slicing=SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25))
    sim.initial_data(InitialData(kind=ID_BRILL_LINDQUIST, punctures=punctures))
    return sim


def richardson_samples(seed: int, n: int = 8, outer: float = 32.0, depth: int = 4, steps: int = 1,
                       pre_steps: int = 0):
    """(features [k][3][512], targets [k], plain indicators [k]) as device tensors for the k leaves of
    one seeded binary configuration after `pre_steps` root steps of its coarse run: that state's tile
    features and plain-criterion indicators, and the log10 Richardson estimate of each leaf's
    truncation error over the next `steps` root steps.  The fine run starts from the same state with
    every leaf refined once (from the analytic initial data when pre_steps is 0, else by the
    tricubic prolongation of the coarse state)."""
    import torch
    punct = binary_punctures(seed)
    coarse = build_sim(n, outer, punct, depth)
    for _ in range(pre_steps):
        coarse.timestep()
    coarse.synchronize()
    feats, ind, leaves = coarse.tile_features()
    feats, ind = feats.clone(), ind.clone()
    if pre_steps == 0:
        fine = build_sim(n, outer, punct, depth, extra_levels=1)
    else:
        fine = build_sim(n, outer, punct, depth)
        nf = 24
        for f in range(nf):
            for buf in (Sim.OLD_STATE, Sim.NEW_STATE):
                fine.tensor(buf, f).copy_(coarse.tensor(buf, f))
        torch.cuda.synchronize()
        fine.add_nodes([s for s in leaves for _ in range(8)], [o for _ in leaves for o in range(8)])
    for _ in range(steps):
        coarse.timestep()
        fine.timestep()
    coarse.synchronize()
    fine.synchronize()
    cs, fs = coarse.state(), fine.state()
    t = n + 6
    fields = (F_CHI, F_ALPHA)
    cdat = [coarse.tensor(Sim.NEW_STATE, f)[: cs["used_slots"] * t ** 3].view(-1, t, t, t)[:, 3:3 + n, 3:3 + n, 3:3 + n]
            for f in fields]
    fdat = [fine.tensor(Sim.NEW_STATE, f)[: fs["used_slots"] * t ** 3].view(-1, t, t, t)[:, 3:3 + n, 3:3 + n, 3:3 + n]
            for f in fields]
    # the fine run's children of each coarse leaf (same slots for the shared part of the tree: the fine
    # tree is built by the same calls followed by one more level)
    fch = fs["children"]
    targets = torch.empty(len(leaves), dtype=torch.float32, device="cuda")
    h = n // 2
    for i, s in enumerate(leaves):
        err = torch.zeros((), device="cuda")
        for cd, fd in zip(cdat, fdat):
            block = torch.empty((n, n, n), device="cuda")
            for o in range(8):
                k = int(fch[8 * s + o])
                child = fd[k]
                # 2x2x2 means of the child's cells -> the coarse cells of octant o
                m = child.reshape(h, 2, h, 2, h, 2).mean(dim=(1, 3, 5))
                ox, oy, oz = o & 1, (o >> 1) & 1, (o >> 2) & 1
                block[oz * h:(oz + 1) * h, oy * h:(oy + 1) * h, ox * h:(ox + 1) * h] = m
            diff = (cd[s] - block).abs().max()
            err = torch.maximum(err, diff)
        targets[i] = torch.log10(err * 16.0 / 15.0 + 1e-12)
    coarse.close()
    fine.close()
    return feats, targets, ind


def train(est: Estimator, feats, targets, epochs: int = 200, batch: int = 64, lr: float = 2e-3, seed: int = 0) -> list:
    """Adam over shuffled mini-batches; returns the mean loss of each epoch."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = feats.shape[0]
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(feats.device)
        tot, cnt = 0.0, 0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            loss = est.train_step(feats[idx], targets[idx], lr)
            tot += loss * len(idx)
            cnt += len(idx)
        losses.append(tot / cnt)
    return losses


def captured_error(scores, targets, k: int) -> float:
    """Share of the total Richardson error (10**targets) held by the k leaves with the highest scores:
    how much of the error a refinement budget of k leaves removes when spent by this ranking."""
    import torch
    err = torch.pow(10.0, targets.double())
    top = torch.topk(scores.double(), k).indices
    return float(err[top].sum() / err.sum())


def calibrate(indicators, targets) -> tuple[float, float]:
    """(a, b) of the least-squares line targets ~ a + b log10(indicators)."""
    import torch
    x = torch.log10(indicators.double() + 1e-12)
    X = torch.stack([torch.ones_like(x), x], 1)
    coef = torch.linalg.lstsq(X, targets.double()[:, None]).solution[:, 0]
    return float(coef[0]), float(coef[1])


def training_set(seeds, n: int = 16, outer: float = 32.0, depth: int = 4, dropped: list | None = None,
                 pre_steps=(0,)):
    """Concatenated (features, targets, indicators) of richardson_samples over the seeds, each at
    every start time in pre_steps.  A sample set that is not all finite (a run that diverged) is
    left out and its (seed, pre_steps) appended to `dropped`."""
    import torch
    fs, ts, inds = [], [], []
    for seed, k in [(seed, k) for seed in seeds for k in pre_steps]:
        f, t, i = richardson_samples(seed, n=n, outer=outer, depth=depth, pre_steps=k)
        if not (bool(torch.isfinite(f).all()) and bool(torch.isfinite(t).all()) and bool(torch.isfinite(i).all())):
            if dropped is not None:
                dropped.append((seed, k))
            continue
        fs.append(f)
        ts.append(t)
        inds.append(i)
    return torch.cat(fs), torch.cat(ts), torch.cat(inds)


def train_default(n_seeds: int = 64, held_out: int = 8, n: int = 16, outer: float = 32.0, depth: int = 4,
                  epochs: int = 60, batch: int = 64, lr: float = 2e-3, pre_steps=(0, 8), log=None):
    """The binary-puncture configuration's network: Richardson samples of n_seeds seeded jittered
    configurations at the start times pre_steps (the last held_out seeds kept for validation), Adam
    on the GPU.  Returns (estimator, calibration (a, b) of the plain indicator on the training
    samples, metadata)."""
    import time
    import torch
    t0 = time.perf_counter()
    train_seeds = list(range(1, n_seeds - held_out + 1))
    val_seeds = list(range(n_seeds - held_out + 1, n_seeds + 1))
    dropped = []
    ft, tt, it = training_set(train_seeds, n, outer, depth, dropped, pre_steps)
    fv, tv, iv = training_set(val_seeds, n, outer, depth, dropped, pre_steps)
    t1 = time.perf_counter()
    est = Estimator(batch, seed=1)
    losses = train(est, ft, tt, epochs=epochs, batch=batch, lr=lr)
    t2 = time.perf_counter()
    a, b = calibrate(it, tt)
    pred = est.forward(fv)
    mse_net = float(((pred - tv) ** 2).mean())
    mse_plain = float(((a + b * torch.log10(iv.double() + 1e-12) - tv.double()) ** 2).mean())
    meta = {"configuration": f"binary Brill-Lindquist, m = 0.5 at x = +-3, jitter 0.01; {n}^3 tiles, "
                             f"root edge {outer}, refined to depth {depth} around the punctures",
            "start_root_steps": list(pre_steps), "train_seeds": len(train_seeds),
            "diverged_samples_left_out": dropped, "train_tiles": int(ft.shape[0]), "val_seeds": len(val_seeds),
            "val_tiles": int(fv.shape[0]), "epochs": epochs, "loss_first": losses[0], "loss_last": losses[-1],
            "val_mse_network": mse_net, "val_mse_calibrated_indicator": mse_plain,
            "val_target_variance": float(tv.var()), "target_quantiles": [float(q) for q in torch.quantile(
                tt, torch.tensor([0.5, 0.8, 0.9], device=tt.device))],
            "seconds_samples": t1 - t0, "seconds_training": t2 - t1}
    if log:
        log(f"estimator: {meta}")
    return est, (a, b), meta


def save(path: str, est: Estimator, calib, meta: dict) -> None:
    import json
    np.savez(path, params=est.get_params(), calibration=np.array(calib, np.float64),
             meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def load_trained(path: str, max_batch: int = 256):
    """(estimator, calibration, metadata) from a file written by save()."""
    import json
    d = np.load(path)
    est = Estimator(max_batch, seed=1)
    est.set_params(d["params"])
    return est, tuple(float(v) for v in d["calibration"]), json.loads(bytes(d["meta"]).decode())


if __name__ == "__main__":
    import argparse
    import sys
    ap = argparse.ArgumentParser(description="train the binary-puncture refinement estimator on the GPU")
    ap.add_argument("--out", required=True)
    ap.add_argument("--seeds", type=int, default=64)
    ap.add_argument("--held-out", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=60)
    a = ap.parse_args()
    e, c, m = train_default(a.seeds, a.held_out, epochs=a.epochs,
                            log=lambda s: print(s, file=sys.stderr, flush=True))
    save(a.out, e, c, m)
    print(m)
