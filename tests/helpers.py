"""Shared test helpers: golden fixtures, error metrics, oracle systems."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def rel_err(F, Fref):
    """Per-particle relative force error |F - Fref| / |Fref|."""
    F = np.asarray(F).reshape(-1, 3)
    Fref = np.asarray(Fref).reshape(-1, 3)
    return np.linalg.norm(F - Fref, axis=1) / np.maximum(np.linalg.norm(Fref, axis=1), 1e-300)


def err_stats(F, Fref):
    e = rel_err(F, Fref)
    return {"p50": float(np.percentile(e, 50)), "p99": float(np.percentile(e, 99)), "max": float(e.max())}


def port_params(pyoracle, is_periodic=0, L=0.0, rsim=0.0, cosmology=0, comoving=0, mius=0.0, h0=0.0, oml=0.0):
    return pyoracle.make_params(is_periodic, L, rsim, cosmology, comoving, mius, h0, oml)
