"""Generate tests/golden/golden.npz from the reference's own builtin library.

Run where the HorsePower sources exist:
    make -C oracle ref            # builds oracle/_ref/libref.so from the sources
    python tests/golden/make_golden.py
Every case in cases.py is run through libref.so (the reference library built
from src/horseir/v3 with its make.sh file set); inputs and outputs are stored.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from horsepower_gb300.abi import Builtins  # noqa: E402
import cases as C  # noqa: E402
import runner  # noqa: E402


def main():
    ref = Builtins(os.path.join(ROOT, "oracle", "_ref", "libref.so"), "reference")
    out = {}
    for case in C.build_cases():
        if case["error"]:
            rc = ref.rc(case["fn"], *[runner.build_arg(ref, a) for a in case["args"]])
            assert rc == case["error"], (case["name"], rc)
            runner.store(case, rc, None, out)
            continue
        rc, obj = runner.run_case(ref, case)
        assert rc == 0, (case["name"], rc)
        runner.store(case, rc, obj, out)
        ref.free_inputs()
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(C.build_cases())} cases")


if __name__ == "__main__":
    main()
