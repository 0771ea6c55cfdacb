"""Step descriptors that lettuce_gb300.native_step builds from lettuce's own
Simulation objects (the drop-in binding lettuce would install at
lettuce/_simulation.py:229), for the simulations of tests/lettuce_cases.py
in float64 and float32: the descriptor with its pointers zeroed, the launch
patterns, the packed flag and no-streaming words made from lettuce's own
masks, and the equilibrium-inlet and MRT tables. tests/test_lettuce_binding.py
checks the mirror classes against them.

    PYTHONPATH=tests/golden/_stubs:<lettuce checkout> \
        python tests/golden/make_binding_golden.py

Output: tests/golden/binding_descriptors.npz
"""
import os
import sys
import warnings

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
warnings.filterwarnings("ignore")

import lettuce  # noqa: E402

import lettuce_gb300  # noqa: E402
from lettuce_cases import cases, step_record  # noqa: E402


def main():
    out = {}
    for tag, dtype in (("f64", torch.float64), ("f32", torch.float32)):
        ctx = lettuce.Context(device="cpu", dtype=dtype, use_native=False)
        for name, sim in cases(lettuce, ctx).items():
            for key, value in step_record(lettuce_gb300.native_step(sim)).items():
                out[f"{tag}/{name}/{key}"] = value
    path = os.path.join(HERE, "binding_descriptors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
