"""Shared helpers for the parity tests: rebuild an oracle case's level-0
description from ``cases.py`` and run it on a backend (oracle or GPU)."""
from __future__ import annotations

import hashlib
import os

import numpy as np

from luma_gb300 import case as hostcase
from tests.golden import cases as CASES

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture(name: str) -> dict:
    with np.load(os.path.join(HERE, f"{name}.npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def level0(name: str) -> hostcase.Level0:
    spec = CASES.CASES[name]
    l0 = hostcase.build_level0(spec["defs"])
    init = CASES.initial_fields(name)
    if init is not None:
        l0.u = init["u"].copy()
    return l0


def initial_state(l0: hostcase.Level0):
    d = l0.defs
    f0 = hostcase.equilibrium(d.dims, d.Q, l0.rho, l0.u).reshape(-1)
    return f0, l0.u.copy(), l0.rho.copy(), l0.force_xyz.copy()
