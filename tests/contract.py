"""The scoring contract the CUDA path is held to against the FP64 oracle.

Energies, within 1e-5 relative:

* |E - E64| <= 1e-5 |E64| on every pose that is not a cancellation case;
* a pose is a cancellation case when its total is under 1% of the sum of the
  absolute values of its pair energies, S > 100 |E64| (FP32 pair terms carry
  about 1e-7 of S each, which cannot resolve 1e-5 of such a total);
* every pose, cancellation cases included, satisfies
  |E - E64| <= 1e-5 max(|E64|, S).

Gradients, each component within 1e-4 relative:

* |G_k - G64_k| <= 1e-4 max(|G64_k|, 0.01 GA_k), where GA_k is the sum of the
  absolute values of the terms that the analytic gradient adds into component
  k (the oracle's orc_grad_scale);
* the floor only acts where a component is under 1% of its own terms (a
  cancellation case, such as a torsion whose moving atoms' forces nearly
  cancel); there the bound is 1e-6 of the terms' scale.

S and GA come from the oracle (mode 3 of orc_score_batch), so the rules do
not depend on the GPU's own numbers.
"""
from __future__ import annotations

from typing import NamedTuple

import numpy as np

E_TOL = 1e-5
G_TOL = 1e-4
CANCEL = 100.0     # S / |E64| above this: a cancellation case
G_FLOOR = 0.01     # fraction of GA_k below which a component is a cancellation case


class Ref(NamedTuple):
    E: np.ndarray
    G: np.ndarray | None
    st: np.ndarray
    S: np.ndarray
    GA: np.ndarray | None


def ref_batch(oracle, system, dofs, grad=False, recenter=False, inter=True, intra=True,
              ph=None, nthreads=16) -> Ref:
    """FP64 energies (and analytic gradients) of the oracle with their
    condition scales S (per pose) and GA (per gradient component)."""
    flags = (oracle.F_INTER if inter else 0) | (oracle.F_INTRA if intra else 0)
    flags |= oracle.F_RECENTER if recenter else 0
    ph = ph if ph is not None else oracle.REF
    dofs = np.ascontiguousarray(dofs, np.float32)
    E, G, st = oracle.score_batch(system.pocket, system.ligand, dofs, flags=flags,
                                  mode=1 if grad else 0, nthreads=nthreads, ph=ph)
    S, GA, _ = oracle.score_batch(system.pocket, system.ligand, dofs, flags=flags, mode=3,
                                  nthreads=nthreads, ph=ph)
    return Ref(E, G, st, S, GA if grad else None)


def energy_errors(E, E64, S) -> dict:
    """Plain relative errors, the cancellation mask and the conditioned
    errors of a batch of energies."""
    E = np.asarray(E, np.float64)
    E64 = np.asarray(E64, np.float64)
    S = np.asarray(S, np.float64)
    d = np.abs(E - E64)
    both_zero = (E64 == 0) & (E == 0)
    cancel = S > CANCEL * np.abs(E64)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(both_zero, 0.0, d / np.abs(E64))
        cond = np.where(both_zero, 0.0, d / np.maximum(np.abs(E64), S))
    keep = ~cancel | both_zero
    return {"rel": rel, "cond": cond, "cancel": cancel & ~both_zero,
            "max_rel": float(rel[keep].max()) if keep.any() else 0.0,
            "max_cond": float(cond.max()) if cond.size else 0.0,
            "n_cancel": int(np.count_nonzero(cancel & ~both_zero))}


def grad_errors(G, G64, GA) -> dict:
    """Per-component errors of a batch of gradients: plain relative, and
    relative to max(|G64_k|, G_FLOOR GA_k)."""
    G = np.asarray(G, np.float64)
    G64 = np.asarray(G64, np.float64)
    GA = np.asarray(GA, np.float64)
    d = np.abs(G - G64)
    den = np.maximum(np.abs(G64), G_FLOOR * GA)
    with np.errstate(divide="ignore", invalid="ignore"):
        comp = np.where(d == 0, 0.0, d / den)
        rel = np.where(d == 0, 0.0, d / np.abs(G64))
    return {"comp": comp, "rel": rel, "max_comp": float(comp.max()) if comp.size else 0.0,
            "max_rel": float(rel.max()) if rel.size else 0.0,
            "frac_plain_ok": float(np.mean(rel <= G_TOL)) if rel.size else 1.0}


def assert_energy(E, E64, S, tol=E_TOL) -> dict:
    r = energy_errors(E, E64, S)
    bad = np.flatnonzero(~r["cancel"] & (r["rel"] > tol))
    assert bad.size == 0, ("plain relative energy error", float(r["rel"][bad].max()), bad[:8])
    assert r["max_cond"] <= tol, ("conditioned energy error", r["max_cond"],
                                  int(np.argmax(r["cond"])))
    return r


def assert_grad(G, G64, GA, tol=G_TOL) -> dict:
    r = grad_errors(G, G64, GA)
    assert r["max_comp"] <= tol, ("gradient component error", r["max_comp"],
                                  np.unravel_index(int(np.argmax(r["comp"])), r["comp"].shape))
    return r


def assert_ref(E, G, ref: Ref, status=None) -> None:
    """Energy (and gradient when ref has one) against an oracle batch."""
    assert_energy(E, ref.E, ref.S)
    if ref.G is not None and G is not None:
        assert_grad(G, ref.G, ref.GA)
    if status is not None:
        assert np.array_equal(np.asarray(status), ref.st)


def fd_check(G, F1, F2, S, GA, h):
    """The gradient G against FP64 central differences F1 (step h) and F2
    (step h / 2), Richardson-extrapolated: R = (4 F2 - F1) / 3.  Only the
    components where the differences are themselves accurate count: their
    truncation error (estimated by |F1 - F2|) and their FP64 rounding (about
    64 eps S / (h / 2), which swamps them where a step moves a huge energy by
    less than its last bits) both under 1e-5 of max(|R|, G_FLOOR GA).
    Returns (errors relative to that, the mask of counted components)."""
    G = np.asarray(G, np.float64)
    R = (4.0 * F2 - F1) / 3.0
    den = np.maximum(np.abs(R), G_FLOOR * GA)
    rounding = 64 * np.finfo(np.float64).eps * np.asarray(S)[:, None] / (h / 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        trusted = (np.abs(F1 - F2) <= 1e-5 * den) & (rounding <= 1e-5 * den) & (den > 0)
        err = np.where(trusted, np.abs(G - R) / den, 0.0)
    return err, trusted
