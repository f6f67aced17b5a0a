"""Seeded synthetic workloads of the forward-path benchmarks.

All data is generated: nested icosphere heads, dipoles uniform in r < 0.8 with
unit moments uniform on the sphere, EEG electrodes on Fibonacci points of the
unit sphere and radial point magnetometers on a Fibonacci lattice.

  config0  3 layers ico3 (642 v / 1280 t each), r .87/.92/1, sigma 1/.0125/1,
           N = 4486, 200 dipoles, 64 EEG (the reference sample head Head3 size)
  config1  3 layers ico4 (2562 v / 5120 t), radii perturbed by a degree<=4
           spherical-harmonic field of 2% amplitude, N = 17926, 2000 dipoles,
           64 EEG, 151 MEG at r = 1.2
  config2  config1 geometry, 500 dipoles, conductivities sampled
           log-uniformly within x[0.5, 2] of nominal
  config3  32 heads of uneven size (ico3/ico4 surfaces, 3 or 4 layers, inner
           radii jittered +-3%), 100-1000 dipoles each, 64 EEG
  config4  4 layers ico5 (10242 v / 20480 t), r .85/.88/.92/1,
           sigma .33/1.79/.0042/.33, N = 102408, 10000 dipoles, 256 EEG, 306 MEG
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import synthetic as syn

SEED = 20261203


@dataclass
class Workload:
    name: str
    head: syn.NestedHead
    dipoles: np.ndarray
    electrodes: np.ndarray
    squids: np.ndarray


def config0(n_dipoles: int = 200) -> Workload:
    head = syn.nested_head(3, [0.87, 0.92, 1.0], [1.0, 0.0125, 1.0])
    return Workload("config0", head, syn.random_dipoles(n_dipoles, SEED + 1),
                    syn.fibonacci_points(64, 1.0), syn.radial_magnetometers(32, 1.2))


def config1(n_dipoles: int = 2000) -> Workload:
    head = syn.nested_head(4, [0.87, 0.92, 1.0], [1.0, 0.0125, 1.0], perturb_seed=SEED + 2)
    return Workload("config1", head, syn.random_dipoles(2000, SEED + 3)[:n_dipoles],
                    syn.fibonacci_points(64, 1.0), syn.radial_magnetometers(151, 1.2))


def config2(n_dipoles: int = 500, base: str = "config1") -> Workload:
    """config1's geometry (or `base`'s, e.g. config0 for a small profiling case)
    with conductivities sampled log-uniformly within x[0.5, 2] of nominal."""
    w = config1(n_dipoles) if base == "config1" else config0(n_dipoles)
    rng = np.random.default_rng(SEED + 4)
    sig = [d[2] for d in w.head.domains]
    new = []
    for (name, b, s) in w.head.domains:
        new.append((name, b, s * float(np.exp(rng.uniform(np.log(0.5), np.log(2.0)))) if s > 0 else 0.0))
    w.head.domains = new
    w.name = "config2"
    return w


def config3_models(n_models: int = 32):
    rng = np.random.default_rng(SEED + 5)
    models = []
    for k in range(n_models):
        L = int(rng.integers(3, 5))
        subdivs = [int(rng.integers(3, 5)) for _ in range(L)]
        base = [0.87, 0.92, 1.0] if L == 3 else [0.85, 0.88, 0.92, 1.0]
        while True:   # jitter the inner radii by +-3%, keeping the surfaces nested 0.02 apart
            radii = [r * (1.0 + rng.uniform(-0.03, 0.03)) for r in base[:-1]] + [1.0]
            if all(radii[i + 1] - radii[i] >= 0.02 for i in range(L - 1)):
                break
        sig = []
        for i in range(L):
            skull = (i == L - 2)
            lo, hi = (0.005, 0.05) if skull else (0.2, 2.0)
            sig.append(float(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        head = syn.nested_head(subdivs, radii, sig)
        nd = int(rng.integers(100, 1001))
        models.append(Workload(f"config3_{k}", head, syn.random_dipoles(nd, SEED + 100 + k, rmax=0.8 * radii[0] / 0.87),
                               syn.fibonacci_points(64, 1.0), np.zeros((0, 6))))
    return models


def batch_small() -> list:
    """Four seconds-scale heads of uneven size for batched-forward tests:
    3 and 4 layers, ico1/ico2, one with SH-perturbed surfaces, one with MEG."""
    out = []
    specs = [(2, [0.87, 0.92, 1.0], [1.0, 0.0125, 1.0], None, 7, True),
             (2, [0.85, 0.88, 0.92, 1.0], [0.33, 1.79, 0.0042, 0.33], None, 12, False),
             (1, [0.80, 0.90, 1.0], [0.5, 0.02, 0.8], None, 5, False),
             (2, [0.87, 0.92, 1.0], [1.2, 0.01, 0.9], SEED + 9, 9, True)]
    for k, (sub, radii, sig, pert, nd, meg) in enumerate(specs):
        head = syn.nested_head(sub, radii, sig, perturb_seed=pert)
        out.append(Workload(f"batch_small_{k}", head, syn.random_dipoles(nd, SEED + 200 + k, rmax=0.7),
                            syn.fibonacci_points(12 + 4 * k, 1.0),
                            syn.radial_magnetometers(10, 1.2) if meg else np.zeros((0, 6))))
    return out


def config4(n_dipoles: int = 10000) -> Workload:
    head = syn.nested_head(5, [0.85, 0.88, 0.92, 1.0], [0.33, 1.79, 0.0042, 0.33])
    return Workload("config4", head, syn.random_dipoles(10000, SEED + 6)[:n_dipoles],
                    syn.fibonacci_points(256, 1.0), syn.radial_magnetometers(306, 1.15))


def small(subdiv: int = 1, n_dipoles: int = 8, layers: int = 3, inward: bool = True, perturb: bool = False) -> Workload:
    """A seconds-scale case for parity tests."""
    if layers == 3:
        head = syn.nested_head(subdiv, [0.87, 0.92, 1.0], [1.0, 0.0125, 1.0], inward=inward,
                               perturb_seed=(SEED + 7) if perturb else None)
    else:
        head = syn.nested_head(subdiv, [0.85, 0.88, 0.92, 1.0], [0.33, 1.79, 0.0042, 0.33], inward=inward,
                               perturb_seed=(SEED + 7) if perturb else None)
    return Workload(f"small_ico{subdiv}_{layers}l", head, syn.random_dipoles(n_dipoles, SEED + 8, rmax=0.75),
                    syn.fibonacci_points(16, 1.0), syn.radial_magnetometers(10, 1.2))
