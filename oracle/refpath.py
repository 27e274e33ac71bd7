"""Where the MatPL source tree is mounted (test infrastructure only).

The golden-fixture scripts under tests/golden/ and the reference-operator recipe
(oracle/ref_build.py) read the reference from ``$MATPL_REF`` when it is set, else from a
``reference`` directory beside this repository's root.  Nothing on the GPU machine, in the tests or
in the benchmark reads it.
"""
import os

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_root() -> str:
    env = os.environ.get("MATPL_REF")
    return env if env else os.path.join(os.path.dirname(REPO), "reference")
