"""Learned proposal for analysis-by-synthesis fitting.

A small CNN -- five 3x3 stride-2 convolutions (3 -> 32 -> 64 -> 128 -> 256
-> 256 channels) and a two-layer MLP (16384 -> 1024 -> 193) -- regresses the
morphable-model, pose and SH parameters of gvr.fitting from a 256 x 256
render: the fitting views rendered at 128 x 128 and tiled 2 x 2.  Every
matrix product of its forward and backward runs on the tcgen05 tensor-core
GEMM (gvr.tc).  It is trained only on renders this rasteriser produces from
parameters drawn as gvr.fitting.sample_params draws them; at test time its
prediction initialises the fit, and the plain fit from the mean takes over
for any element whose photometric RMSE is still above a threshold after a
few steps.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import fitting, tc
from .fitting import N_PARAMS, PARAM_SLICES

CHANNELS = (3, 32, 64, 128, 256, 256)
HIDDEN = 1024        # MLP width; held-out shape / albedo error after 800 steps 0.73 / 0.74 (512: 0.77 / 0.80)
INPUT = 256          # network input edge (2 x 2 views of VIEW pixels)
VIEW = 128


def param_stats():
    """Mean and scale of every parameter under sample_params; scale 0 marks
    parameters that sample_params keeps fixed (roll, pitch, translation)."""
    mu = np.zeros(N_PARAMS, np.float32)
    sd = np.ones(N_PARAMS, np.float32)
    sd[160:166] = 0.0
    sd[161] = math.radians(45.0) / math.sqrt(3.0)       # yaw U[-45, 45] deg
    sh = PARAM_SLICES["sh"]
    sd[sh] = 0.1
    for k in (166, 175, 184):                            # band 0 U[0.5, 1.2]
        mu[k] = 0.85
        sd[k] = 0.7 / math.sqrt(12.0)
    return mu, sd


class ProposalNet:
    """FP32 master weights (He-initialised); BF16 on the tensor cores."""

    def __init__(self, device, seed=0):
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.device = torch.device(device)
        self.convs = []
        for cin, cout in zip(CHANNELS[:-1], CHANNELS[1:]):
            w = torch.randn(cout, 9 * cin, generator=g) * math.sqrt(2.0 / (9 * cin))
            self.convs.append((w.to(self.device).requires_grad_(True),
                               torch.zeros(cout, device=self.device, requires_grad=True)))
        feat = CHANNELS[-1] * (INPUT // 32) ** 2
        w1 = torch.randn(HIDDEN, feat, generator=g) * math.sqrt(2.0 / feat)
        w2 = torch.randn(N_PARAMS, HIDDEN, generator=g) * math.sqrt(1.0 / HIDDEN)
        self.fc = [(w1.to(self.device).requires_grad_(True), torch.zeros(HIDDEN, device=self.device, requires_grad=True)),
                   (w2.to(self.device).requires_grad_(True), torch.zeros(N_PARAMS, device=self.device,
                                                                         requires_grad=True))]
        mu, sd = param_stats()
        self.mu = torch.from_numpy(mu).to(self.device)
        self.sd = torch.from_numpy(sd).to(self.device)

    def parameters(self):
        return [t for pair in self.convs + self.fc for t in pair]

    def __call__(self, x):
        """x: [B, 256, 256, 3] renders -> [B, 193] normalised parameters."""
        h = (x - 0.5).to(torch.bfloat16).contiguous()
        for w, b in self.convs:
            h = tc.Conv3x3s2.apply(h, w, b)
        h = h.reshape(h.shape[0], -1)
        h = tc.Linear.apply(h, self.fc[0][0], self.fc[0][1], True)
        return tc.Linear.apply(h, self.fc[1][0], self.fc[1][1], False)

    def predict(self, x):
        """Denormalised parameters [B, 193] (fixed parameters at their value)."""
        with torch.no_grad():
            return self.mu + self(x) * self.sd

    def state(self):
        return [t.detach().cpu() for t in self.parameters()]

    def load(self, state):
        with torch.no_grad():
            for t, s in zip(self.parameters(), state):
                t.copy_(s.to(self.device))


def mosaic(views):
    """[B, 4, h, w, 3] -> [B, 2h, 2w, 3]."""
    B, C, h, w, _ = views.shape
    return views[:, :4].reshape(B, 2, 2, h, w, 3).permute(0, 1, 3, 2, 4, 5).reshape(B, 2 * h, 2 * w, 3)


class Trainer:
    """Trains a ProposalNet on renders of random parameters, drawn fresh for
    every batch (so `steps * batch` renders in all)."""

    def __init__(self, model: fitting.MorphableModel, net: ProposalNet, batch=256, lr=1e-3, seed=1):
        self.model, self.net, self.batch = model, net, batch
        self.view_fitter = fitting.Fitter(model, num_views=4, size=VIEW)
        self.rng = np.random.default_rng(seed)
        self.opt = torch.optim.Adam(net.parameters(), lr=lr)
        self.base_lr = [g["lr"] for g in self.opt.param_groups]
        self.steps_done = 0
        self.active = (net.sd > 0).float()

    def sample(self, B):
        gt = fitting.sample_params(self.rng, B)
        p = torch.from_numpy(gt).to(self.model.device)
        with torch.no_grad():
            x = mosaic(self.view_fitter.render(p))
        return p, x

    def step(self):
        p, x = self.sample(self.batch)
        target = (p - self.net.mu) / torch.where(self.net.sd > 0, self.net.sd, torch.ones_like(self.net.sd))
        out = self.net(x)
        loss = (((out - target) ** 2) * self.active).sum(1).mean() / self.active.sum()
        self.opt.zero_grad(set_to_none=True)
        loss.backward()
        self.opt.step()
        return loss

    def train(self, steps, log_every=0, lr_final=0.05, start=0):
        """Adam with the step size decaying geometrically to lr_final times
        its start over `steps`, running steps start..steps-1 (start > 0
        continues a run restored by resume()); returns (losses, seconds)."""
        base = self.base_lr
        losses = []
        t0 = time.perf_counter()
        for k in range(start, steps):
            for g, b in zip(self.opt.param_groups, base):
                g["lr"] = b * lr_final ** (k / max(steps, 1))
            loss = self.step()
            self.steps_done = k + 1
            if log_every and (k % log_every == 0 or k == steps - 1):
                losses.append((k, float(loss.detach())))
        torch.cuda.synchronize()
        return losses, time.perf_counter() - t0

    def checkpoint(self, path):
        """Weights, Adam state, the parameter sampler's RNG state and the
        steps done, to `path` (torch.save)."""
        torch.save({"weights": self.net.state(), "opt": self.opt.state_dict(), "base_lr": self.base_lr,
                    "rng": self.rng.bit_generator.state, "steps_done": self.steps_done}, path)

    def resume(self, path):
        """Restores a checkpoint(); train(steps, start=self.steps_done) then
        continues the run where it stopped."""
        ck = torch.load(path, map_location="cpu", weights_only=False)
        self.net.load(ck["weights"])
        self.opt.load_state_dict(ck["opt"])
        self.base_lr = list(ck["base_lr"])
        self.rng.bit_generator.state = ck["rng"]
        self.steps_done = int(ck["steps_done"])


def evaluate(fitter: fitting.Fitter, net: ProposalNet | None, seeds, steps=200, goal=0.01, fallback_step=20,
             fallback_rmse=0.05, batch=50):
    """Fits the targets of `seeds` (held-out parameter draws) from the
    proposal (with the plain fit as fallback; refinement step sizes
    Fitter.LR) or, with net=None, from the mean (step sizes
    Fitter.LR_FROM_MEAN, which suit a far start).  Returns per-seed steps and
    GPU ms to RMSE <= goal (None if never), the final RMSE, and the total GPU
    ms (all batches)."""
    view_fitter = fitting.Fitter(fitter.model, num_views=4, size=VIEW) if net is not None else None
    steps_to, ms_to, final, curves, step_ms = [], [], [], [], []
    total_ms = 0.0
    for i in range(0, len(seeds), batch):
        chunk = seeds[i:i + batch]
        gt = np.concatenate([fitting.sample_params(np.random.default_rng(int(s)), 1) for s in chunk])
        p = torch.from_numpy(gt).to(fitter.model.device)
        with torch.no_grad():
            target = fitter.render(p)
        mean = fitting.mean_params(len(chunk))
        if net is None:
            res = fitter.fit(target, mean, steps=steps, goal=goal, lr=fitting.Fitter.LR_FROM_MEAN)
            extra_ms = 0.0
        else:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            with torch.no_grad():
                x = mosaic(view_fitter.render(p))       # the observation the network sees
                init = net.predict(x).cpu().numpy()
            e1.record()
            e1.synchronize()
            extra_ms = e0.elapsed_time(e1)
            res = fitter.fit(target, init, steps=steps, goal=goal, fallback=(fallback_step, fallback_rmse, mean))
        total_ms += res.gpu_ms + extra_ms
        for j in range(len(chunk)):
            steps_to.append(res.steps_to_goal[j])
            ms_to.append(None if res.gpu_ms_to_goal[j] is None else res.gpu_ms_to_goal[j] + extra_ms)
            final.append(float(res.rmse[-1, j]))
            curves.append(res.rmse[:, j])
            step_ms.append((res.step_ms + extra_ms) / len(chunk))
    return dict(steps_to_goal=steps_to, gpu_ms_to_goal=ms_to, final_rmse=final, total_gpu_ms=total_ms,
                rmse_curves=curves, step_ms_per_fit=step_ms)


def time_to_match(learned, plain):
    """Per seed: GPU ms (per fit) the learned fit needs to reach the RMSE the
    plain fit ends with, and the plain fit's whole GPU ms; seeds the learned
    fit never matches count with its whole run."""
    t_l, t_p = [], []
    for cl, ml, cp, mp in zip(learned["rmse_curves"], learned["step_ms_per_fit"], plain["rmse_curves"],
                              plain["step_ms_per_fit"]):
        hit = np.nonzero(cl <= cp[-1])[0]
        t_l.append(float(ml[hit[0]]) if hit.size else float(ml[-1]))
        t_p.append(float(mp[-1]))
    return np.array(t_l), np.array(t_p)
