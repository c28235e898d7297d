"""Learned row marking: trace collection and GPU training of the marking MLP.

The pipeline the library supports end to end:

    traces = collect_traces(mips)                    # the propagator logs its own rounds
    model, t, info = train_marking_model(*traces)    # GPU forward/backward kernels, Adam
    ctx.set_model(model, t, info["min_len"])         # learned rounds; a FULL or FLUSH round
                                                     # without change certifies the fixpoint

Labels are "processing this marked row tightened a bound". The model decides
only for rows of at least `min_len` non-zeros (shorter rows are always
processed: they are cheap, and deferring a productive one stalls a propagation
front), so it is trained on those rows only, each weighted by its length (the
work a deferral saves) with both classes weighing the same. The logit
threshold is the largest one that keeps `recall` of the productive training
rows selected: deferring a productive row delays propagation, deferring an
unproductive one lets its markings coalesce into one later processing.
"""
from __future__ import annotations

from typing import Iterable, Tuple

import numpy as np

import gdp


def collect_traces(mips: Iterable[gdp.MIP], capacity: int = 4_000_000, sync_type: int = gdp.MEGAKERNEL,
                   max_rounds: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    """Trace propagations (exact marking) of every MIP: features [k, 16], labels [k]."""
    xs, ys = [], []
    for mip in mips:
        with gdp.Context(mip, sync_type=sync_type, max_rounds=max_rounds) as ctx:
            x, y, *_ = ctx.trace(capacity=capacity)
        xs.append(x)
        ys.append(y)
    if not xs:
        return np.zeros((0, gdp.MLP_FEATURES), np.float32), np.zeros(0, np.float32)
    return np.concatenate(xs), np.concatenate(ys)


def row_length(x: np.ndarray) -> np.ndarray:
    """Row length from feature 0 (log2(1 + len) / 16)."""
    return np.rint(np.exp2(16.0 * x[:, 0].astype(np.float64)) - 1.0)


def balanced_weights(y: np.ndarray, cost: np.ndarray | None = None) -> np.ndarray:
    c = np.ones(len(y)) if cost is None else cost / max(np.mean(cost), 1e-12)
    wp, wn = np.sum(c[y > 0.5]), np.sum(c[y <= 0.5])
    if wp == 0 or wn == 0:
        return c.astype(np.float32)
    return np.where(y > 0.5, 0.5 * c * len(y) / wp, 0.5 * c * len(y) / wn).astype(np.float32)


def recall_threshold(z: np.ndarray, y: np.ndarray, recall: float) -> float:
    """Largest logit threshold selecting at least `recall` of the positive samples."""
    zp = np.sort(z[y > 0.5])
    if zp.size == 0:
        return 0.0
    k = int(np.floor((1.0 - recall) * zp.size))
    return float(zp[min(max(k, 0), zp.size - 1)])


def train_marking_model(x: np.ndarray, y: np.ndarray, epochs: int = 6, batch: int = 8192, lr: float = 2e-3,
                        seed: int = 0, recall: float = 0.98, min_len: int = 8, device: int = 0):
    """Trains an Mlp on the trace samples of rows with at least `min_len`
    non-zeros, on the GPU. Returns (model, threshold, info); attach with
    ctx.set_model(model, threshold, min_len)."""
    model = gdp.Mlp(seed=seed, device=device)
    keep = row_length(x) >= min_len
    xk, yk = x[keep], y[keep]
    info = {"samples": int(len(y)), "samples_trained": int(len(yk)), "min_len": int(min_len),
            "positive_rate": float(np.mean(yk)) if len(yk) else 0.0}
    if len(yk) == 0:
        info.update(loss=0.0, threshold=-1e30, recall=1.0, selected_rate=1.0)
        return model, -1e30, info
    w = balanced_weights(yk, row_length(xk))
    loss = model.train(xk, yk, w, epochs=epochs, batch=batch, lr=lr, seed=seed + 1)
    z = model.forward(xk)
    tau = recall_threshold(z, yk, recall) if np.any(yk > 0.5) else float(np.max(z)) + 1.0
    sel = z >= tau
    info.update(loss=loss, threshold=tau, recall=float(np.mean(sel[yk > 0.5])) if np.any(yk > 0.5) else 1.0,
                selected_rate=float(np.mean(sel)))
    return model, tau, info
