"""Replay of detected photons and the Jacobians built on it.

A detected photon is re-traced from its saved 16-byte RNG state; since its
random stream, the mesh and the optical properties are unchanged, it follows
the same path (the engine is deterministic per photon) and reaches the same
detector.  During the replay the engine deposits, per element:

* ``wl``: replay weight x path length  (src/mmc_core.cl:814-818)
* ``wp``: replay weight x path length x mus / slen0  (src/mmc_core.cl:819-829),
  the reference's estimator of the scattering-event share of an element
* ``wn``: replay weight once per scattering event in the element where it
  happens (exact scatter counts; no reference counterpart)

For a detected photon p with weight w_p = w0 exp(-sum_e mua_e L_pe) and n_pe
scattering events in element e, the likelihood-ratio derivatives are
    dw_p/dmua_e = -w_p L_pe,      dw_p/dmus_e = w_p (n_pe / mus_e - L_pe),
so with replay weight = w_p (or any per-photon factor times w_p):
    J_mua = -wl,    J_mus = wn / mus - wl.
The reference builds the same Jacobians in matlab/mmcjmua.m:57 (Jmua = -wl)
and matlab/mmcjmus.m:36-69 (Jmus = Jmua + wp/mus).

``ReplayLoss`` is the torch.autograd.Function of the differentiable
detector-weight loss L = sum_d c_d log W_d.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from .core import Mesh, SimConfig, simulate, simulate_batch

R_C0 = np.float32(3.335640951981520e-12)


def detected_weight(detp: np.ndarray, media: np.ndarray, unitinmm: float = 1.0) -> np.ndarray:
    """w0 * exp(-sum_i mua_i * L_i) of each record (columns: detid, nscat[M],
    ppath[M], ..., w0) -- src/mmc_utils.c:3620-3625 (float32 arithmetic)."""
    M = media.shape[0] - 1
    pp = detp[:, 1 + M:1 + 2 * M].astype(np.float32)
    w = np.ones(len(detp), np.float32)
    for j in range(M):
        w = w * np.exp(np.float32(-media[j + 1, 0]) * pp[:, j] * np.float32(unitinmm)).astype(np.float32)
    return w


def replay_inputs(detp: np.ndarray, seeds: np.ndarray, media: np.ndarray, replaydet: int = 0,
                  tstart: float = 0.0, tend: float = 1.0, unitinmm: float = 1.0):
    """Selects the photons to replay and computes their weights and arrival
    times as the reference's mcx_replayinit does (src/mmc_utils.c:3577-3638):
    photons of detector `replaydet` (all if <= 0) whose time of flight lies in
    [tstart, tend].  Returns (seeds (n,2) uint64, weight, time, index)."""
    M = media.shape[0] - 1
    ids = detp[:, 0].astype(np.int64)
    keep = np.ones(len(detp), bool) if replaydet <= 0 else (ids == replaydet)
    pp = detp[:, 1 + M:1 + 2 * M].astype(np.float32)
    w = np.ones(len(detp), np.float32)
    t = np.zeros(len(detp), np.float32)
    for j in range(M):
        w = (w * np.exp(np.float32(-media[j + 1, 0]) * pp[:, j])).astype(np.float32)
        t = (t + pp[:, j] * np.float32(unitinmm) * R_C0 * np.float32(media[j + 1, 3])).astype(np.float32)
    keep &= (t >= np.float32(tstart)) & (t <= np.float32(tend))
    idx = np.nonzero(keep)[0]
    s = np.ascontiguousarray(seeds[idx], np.uint8).reshape(len(idx), 16).view(np.uint64).reshape(len(idx), 2)
    return s.copy(), w[idx].copy(), t[idx].copy(), idx


def replay(mesh: Mesh, cfg: SimConfig, detp: np.ndarray, seeds: np.ndarray, outputtype: str = "wl",
           replaydet: int = 0, weight: Optional[np.ndarray] = None, normalize: bool = False):
    """Re-traces the detected photons (optionally with custom per-photon replay
    weights) and returns the SimResult of the replay (`field` holds the
    requested deposits, raw unless `normalize`)."""
    s, w, t, idx = replay_inputs(detp, seeds, np.asarray(cfg.media), replaydet, cfg.tstart, cfg.tend, cfg.unitinmm)
    if weight is not None:
        w = np.asarray(weight, np.float32)[idx] if len(weight) == len(detp) else np.asarray(weight, np.float32)
    rcfg = dataclasses.replace(cfg, nphoton=len(idx), replayseed=s, replayweight=w, replaytime=t,
                               outputtype=outputtype, isnormalized=1 if normalize else 0, basisorder=0,
                               photon_offset=0, save_field=True)
    return simulate(mesh, rcfg), idx


def jacobians(mesh: Mesh, cfg: SimConfig, detp: np.ndarray, seeds: np.ndarray, replaydet: int = 0,
              coef: Optional[np.ndarray] = None):
    """(J_mua, J_mus) per element and gate, for sum over the replayed photons of
    coef_p * w_p (coef = 1 gives the detected weight of `replaydet`)."""
    w = detected_weight(detp, np.asarray(cfg.media), cfg.unitinmm).astype(np.float64)
    if coef is not None:
        w = w * np.asarray(coef, np.float64)
    # both replays (path lengths and scatter counts) share one batched launch
    s, _, t, idx = replay_inputs(detp, seeds, np.asarray(cfg.media), replaydet, cfg.tstart, cfg.tend, cfg.unitinmm)
    # the replays always return their deposits, whatever the forward configuration saved
    base = dataclasses.replace(cfg, nphoton=len(idx), replayseed=s, replayweight=w[idx].astype(np.float32),
                               replaytime=t, isnormalized=0, basisorder=0, photon_offset=0, save_field=True)
    wl, wn = simulate_batch([mesh, mesh], [dataclasses.replace(base, outputtype="wl"),
                                           dataclasses.replace(base, outputtype="wn")])
    mus = np.asarray(cfg.media, np.float64)[mesh.label, 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        jmus = np.where(mus > 0, wn.field / mus, 0.0) - wl.field
    return -wl.field, jmus


def loss_and_grads(mesh: Mesh, cfg: SimConfig, detp: np.ndarray, seeds: np.ndarray, c: np.ndarray):
    """L = sum_d c_d log W_d over the detected records and its per-element
    derivatives dL/dmua, dL/dmus (summed over gates), from one replay pair:
    each photon replays with weight c_d / W_d * w_p."""
    media = np.asarray(cfg.media)
    w = detected_weight(detp, media, cfg.unitinmm).astype(np.float64)
    ids = detp[:, 0].astype(int)
    ndet = len(c)
    W = np.array([w[ids == d + 1].sum() for d in range(ndet)])
    L = float(np.sum(np.asarray(c) * np.log(W)))
    c = np.asarray(c, np.float64)
    ok = (ids >= 1) & (ids <= ndet)
    coef = np.zeros(len(ids))
    coef[ok] = c[ids[ok] - 1] / W[ids[ok] - 1]
    jmua, jmus = jacobians(mesh, cfg, detp, seeds, 0, coef)
    return L, W, jmua.sum(0), jmus.sum(0)


def _torch():
    import torch
    return torch


class ReplayLoss:
    """torch.autograd.Function wrapper: L(mua, mus) = sum_d c_d log W_d.

    forward runs a forward simulation with per-element optical properties
    taken from the element labels of the mesh and the per-medium tensors
    `mua`, `mus` (shape (nmedia,)); backward replays the detected photons and
    returns dL/dmua, dL/dmus per medium (the per-element Jacobians summed over
    the elements of each medium).  Per-element gradients are available from
    `loss_and_grads`.
    """

    @staticmethod
    def apply(mesh: Mesh, cfg: SimConfig, c, mua, mus):
        torch = _torch()

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, mua_t, mus_t):
                media = np.asarray(cfg.media, np.float32).copy()
                media[:, 0] = mua_t.detach().cpu().numpy()
                media[:, 1] = mus_t.detach().cpu().numpy()
                fcfg = dataclasses.replace(cfg, media=media, issavedet=1, issaveseed=1, save_field=False)
                res = simulate(mesh, fcfg)
                L, W, gmua, gmus = loss_and_grads(mesh, fcfg, res.detp, res.seeds, np.asarray(c, np.float64))
                lab = mesh.label
                nmed = media.shape[0]
                ctx.save_for_backward(torch.tensor(np.bincount(lab, gmua, nmed)),
                                      torch.tensor(np.bincount(lab, gmus, nmed)))
                return torch.tensor(L, dtype=torch.float64)

            @staticmethod
            def backward(ctx, gL):
                gmua, gmus = ctx.saved_tensors
                return gL * gmua, gL * gmus

        return _Fn.apply(mua, mus)
