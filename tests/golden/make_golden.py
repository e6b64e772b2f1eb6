"""Regenerate the golden fixtures of this directory.

Runs every scenario of ``scenarios.py`` through clODE's own kernel sources
compiled as C (``oracle/build.py build_reference``; needs the clODE source
tree: CLODE_REFERENCE_ROOT, else a checkout named ``reference`` beside the
repository) and saves
inputs and outputs as ``<name>.npz``.  Usage: ``python -m tests.golden.make_golden``.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.build import reference_available  # noqa: E402
from tests.golden.scenarios import scenarios  # noqa: E402
from tests.parity import run_oracle  # noqa: E402

OUTPUT_KEYS = ("xf", "tf", "dt", "t", "x", "dx", "n_stored", "x0")


def main():
    if not reference_available():
        sys.exit("clODE sources not found: cannot regenerate the golden fixtures")
    for name, (sc, exact, rtol) in scenarios().items():
        out = run_oracle(sc, nthreads=1, reference=True)
        arrays = {k: out[k] for k in OUTPUT_KEYS if k in out}
        if "F_list" in out:
            arrays["F"] = np.stack(out["F_list"])
        meta = {"exact": exact, "rtol": rtol, "source": "clODE kernels compiled as C (oracle/_ref)"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
