"""Basin classification of walks and connections with three oracle builds.

A Newton walk whose outcome changes under a one-rounding perturbation sits on
a basin boundary: no FP32 implementation can be expected to reproduce it.  The
oracle is built three ways from the same source (oracle/Makefile): FP32 without
FMA contraction (the oracle proper), FP32 with FMA contraction, and FP64.  A
walk (or a connection) is *well conditioned* when all three agree; the GPU is
held to the oracle exactly there, and the fraction that is not well
conditioned is the basin-crossing fraction.

Helper module of the test suite (not collected: no test_ prefix).
"""
from __future__ import annotations

import numpy as np

POS_TOL = 1e-4   # same solution: positions within 1e-4 of scene scale 1


def walk_outcome_equal(a: np.ndarray, b: np.ndarray, rows=slice(2, 5)) -> np.ndarray:
    """Per walk: same converged flag and, when both converged, the same
    solution (rows of the position, within POS_TOL)."""
    oka, okb = a[0] > 0.5, b[0] > 0.5
    d = np.linalg.norm(a[rows] - b[rows], axis=0)
    return (oka == okb) & (~oka | (d < POS_TOL))


def well_conditioned_walks(outs: dict, rows=slice(2, 5)) -> np.ndarray:
    """outs: {"f32": out, "fma": out, "f64": out, ...} of the same walks; every
    member must agree with "f32"."""
    ref = outs["f32"]
    mask = np.ones(ref.shape[1], bool)
    for k, o in outs.items():
        if k != "f32":
            mask &= walk_outcome_equal(ref, o, rows)
    return mask


def leave_one_out_rates(outs: dict, rows=slice(2, 5)) -> dict:
    """For each member m other than "f32": the fraction of walks on which m
    disagrees with "f32" among the walks that every other member calls well
    conditioned.  How often one more one-rounding perturbation of the oracle
    itself flips a walk the rest of the ensemble agrees on: the yardstick for
    the GPU's mismatch on the well-conditioned walks of a chaotic scene."""
    ref = outs["f32"]
    rates = {}
    for m in outs:
        if m == "f32":
            continue
        rest = {k: v for k, v in outs.items() if k != m}
        mask = well_conditioned_walks(rest, rows)
        agree = walk_outcome_equal(outs[m], ref, rows)
        rates[m] = float(np.mean(~agree[mask])) if mask.any() else 0.0
    return rates


def nudge(a: np.ndarray, rows, up: bool = True) -> np.ndarray:
    """A copy of a with the given rows moved by one ulp (up or down): a
    one-rounding perturbation of the inputs."""
    b = np.array(a, np.float32, copy=True)
    b[rows] = np.nextafter(b[rows], np.float32(np.inf if up else -np.inf))
    return b


def connection_equal(a, b, rtol: float = 1e-3) -> np.ndarray:
    """Per query: same unique-solution count, same walk count and values
    within rtol of the query's largest component.  a, b: (value, count,
    walks) triples."""
    va, ca, wa = a[:3]
    vb, cb, wb = b[:3]
    scale = np.maximum(np.abs(vb).max(axis=0), 1e-6)
    rel = np.abs(va - vb).max(axis=0) / scale
    return (ca == cb) & (wa == wb) & (rel <= rtol)


def well_conditioned_connections(outs: dict, rtol: float = 1e-3) -> np.ndarray:
    ref = outs["f32"]
    mask = np.ones(ref[1].shape[0], bool)
    for k, o in outs.items():
        if k != "f32":
            mask &= connection_equal(ref, o, rtol)
    return mask


def leave_one_out_connection_rates(outs: dict, rtol: float = 1e-3) -> dict:
    """leave_one_out_rates for connection outputs (value, count, walks)."""
    ref = outs["f32"]
    rates = {}
    for m in outs:
        if m == "f32":
            continue
        rest = {k: v for k, v in outs.items() if k != m}
        mask = well_conditioned_connections(rest, rtol)
        agree = connection_equal(outs[m], ref, rtol)
        rates[m] = float(np.mean(~agree[mask])) if mask.any() else 0.0
    return rates


def oracle_walks(oracle, desc, fn: str, *args) -> dict:
    """Run one walk-batch method of OracleScene in all three builds."""
    return {v: getattr(oracle.OracleScene(desc, variant=v), fn)(*args) for v in ("f32", "fma", "f64")}


def oracle_connections(oracle, desc, config, queries, **kw) -> dict:
    return {v: oracle.OracleScene(desc, variant=v).connect_batch(config, queries, **kw)
            for v in ("f32", "fma", "f64")}
