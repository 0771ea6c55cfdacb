"""Float64 reference of the 3-D Taylor-Green benchmark: D3Q19 BGK, 256^3
periodic, Re 1600, Ma 0.05, 1000 PRE_STREAMING steps, computed by the CPU
oracle (the C restatement of lettuce's torch step, pinned to vectors that
lettuce itself generated) on every host core. The full field (2.5 GB of
float64 populations) is too large to commit, so the fixture keeps what a
GPU run can be checked against at full size:

* the velocity and density at 8192 cells (a regular 16^3 sub-lattice with
  offset 5, then 4096 seeded random cells);
* per-plane sums: for every velocity component c and axis a, the sums of
  u_c and of u_c^2 over each plane normal to a (3 x 3 x 256 values each;
  the sums of u_c vanish by the vortex's symmetry up to rounding, the sums
  of u_c^2 do not), and the density deviation rho - 1 likewise (3 x 256) --
  every cell of the field enters them;
* float64 totals: mass, sum |u|^2 per component, max |u|^2.

The initial populations come from lettuce's own TaylorGreenVortex (float64,
fneq initialisation) when lettuce is importable, else from this package's
CPU set-up of the same flow; the file records which. With lettuce
importable the script also advances lettuce's torch step by ``--check-steps``
steps at full size and records the largest difference to the oracle after
the same steps (the oracle's pin at this grid size).

    PYTHONPATH=tests/golden/_stubs:<lettuce checkout> \
        python tests/golden/make_accuracy_pin.py [--threads N]

Takes about 20 minutes on 8 x86 cores. Output:
``tests/golden/accuracy_pin_d3q19_256_f64_1000.npz``.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

RES = 256
RE, MA = 1600, 0.05
STEPS = 1000
OUT = os.path.join(HERE, "accuracy_pin_d3q19_256_f64_1000.npz")


def sample_cells(n=RES, seed=7):
    """flat indices of the 8192 sampled cells"""
    g = np.arange(5, n, 16)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    regular = np.ravel_multi_index((X.ravel(), Y.ravel(), Z.ravel()), (n, n, n))
    rng = np.random.default_rng(seed)
    rand = rng.choice(n ** 3, size=4096, replace=False)
    return np.concatenate([regular, np.sort(rand)]).astype(np.int64)


def plane_sums(a):
    """[3 axes, n] sums of a [n, n, n] field over the planes normal to each axis"""
    return np.stack([a.sum(axis=(1, 2)), a.sum(axis=(0, 2)), a.sum(axis=(0, 1))])


def summarise(rho, u):
    cells = sample_cells()
    out = {
        "cells": cells,
        "u_samples": u.reshape(3, -1)[:, cells].copy(),
        "rho_samples": rho.reshape(-1)[cells].copy(),
        "u_plane_sums": np.stack([plane_sums(u[c]) for c in range(3)]),
        "u_sq_plane_sums": np.stack([plane_sums(u[c] * u[c]) for c in range(3)]),
        "rho_plane_sums": plane_sums(rho),
        "drho_plane_sums": plane_sums(rho - 1.0),
        "mass": np.float64(rho.sum()),
        "u_sq_sums": np.array([np.sum(u[c] * u[c]) for c in range(3)]),
        "u_sq_max": np.float64(np.max(np.sum(u * u, axis=0))),
    }
    return out


def initial_field():
    """(f0 float64 [19, 256, 256, 256], tau, source)"""
    import torch
    try:
        import lettuce as lettuce_ref
        ctx = lettuce_ref.Context(device="cpu", dtype=torch.float64, use_native=False)
        flow = lettuce_ref.TaylorGreenVortex(ctx, [RES] * 3, RE, MA, lettuce_ref.D3Q19())
        return (flow.f.numpy().copy(), float(flow.units.relaxation_parameter_lu),
                "lettuce TaylorGreenVortex (float64)", (lettuce_ref, flow))
    except ImportError:
        import lettuce_gb300 as lt
        ctx = lt.Context("cpu", torch.float64)
        flow = lt.TaylorGreenVortex(ctx, [RES] * 3, RE, MA, lt.D3Q19)
        return (flow.f.numpy().copy(), float(flow.units.relaxation_parameter_lu),
                "lettuce_gb300 TaylorGreenVortex, CPU set-up (float64)", None)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--check-steps", type=int, default=3)
    args = ap.parse_args()
    from oracle import oracle as orc
    orc.build()
    f0, tau, source, ref = initial_field()
    print(f"initial field from {source}; tau = {tau!r}", flush=True)

    pin = {}
    if ref is not None and args.check_steps > 0:
        lettuce_ref, flow = ref
        sim = lettuce_ref.Simulation(flow, lettuce_ref.BGKCollision(tau=tau), [],
                                     lettuce_ref.StreamingStrategy.PRE_STREAMING)
        t0 = time.perf_counter()
        sim(args.check_steps)
        t_ref = time.perf_counter() - t0
        f_orc = orc.run("D3Q19", f0, args.check_steps, collision="bgk", tau=tau,
                        strategy="PRE_STREAMING", nthreads=args.threads)
        diff = float(np.max(np.abs(flow.f.numpy() - f_orc)))
        pin = {"lettuce_check_steps": np.int64(args.check_steps),
               "lettuce_check_max_abs_diff": np.float64(diff)}
        print(f"lettuce vs oracle after {args.check_steps} steps at 256^3: max |df| = {diff:.3e}"
              f" (lettuce took {t_ref:.1f} s)", flush=True)
        del f_orc, sim, flow
    t0 = time.perf_counter()
    f = orc.run("D3Q19", f0, STEPS, collision="bgk", tau=tau, strategy="PRE_STREAMING",
                nthreads=args.threads)
    dt = time.perf_counter() - t0
    print(f"oracle: {STEPS} steps in {dt:.0f} s ({STEPS * RES ** 3 / dt / 1e6:.1f} MLUPS)",
          flush=True)
    del f0
    rho, u = orc.moments("D3Q19", f, nthreads=args.threads)
    del f
    s = summarise(rho, u)
    np.savez_compressed(OUT, grid=np.int64(RES), steps=np.int64(STEPS), reynolds=np.float64(RE),
                        mach=np.float64(MA), tau=np.float64(tau), source=np.array(source),
                        oracle_seconds=np.float64(dt), threads=np.int64(args.threads),
                        **pin, **s)
    print(f"wrote {OUT}", flush=True)


if __name__ == "__main__":
    main()
