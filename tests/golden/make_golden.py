"""Writes the golden fixtures of tests/golden (see golden_cases.py) with
the oracle: python -m tests.golden.make_golden [case ...]."""
import sys

import numpy as np

from tests.golden import golden_cases as gc


def main(names):
    for name in names or list(gc.CASES):
        d = gc.generate(name)
        np.savez_compressed(gc.path(name), **d)
        print(name, gc.path(name))


if __name__ == "__main__":
    main(sys.argv[1:])
