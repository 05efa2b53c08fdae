"""Extract the reference's Bessel I0 table (tests/bessel.c of the reference:
I0(j) for j = 0, 1, 2, ..., written to 64 digits) into
tests/golden/bessel_i0.npz (float64 values and their exact decimal strings).

Usage: python tests/golden/make_bessel_table.py [reference root]
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402  (the reference checkout's location)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else oracle.REFERENCE_SRC
    with open(os.path.join(root, "tests", "bessel.c")) as fh:
        text = fh.read()
    body = text[text.index("static const R r[]"):]
    body = body[:body.index("};")]
    vals = re.findall(r"K\(([-+0-9.eE]+)\)", body)
    np.savez_compressed(os.path.join(HERE, "bessel_i0.npz"), x=np.arange(len(vals), dtype=np.float64),
                        i0=np.array([float(v) for v in vals]), text=np.array(vals))
    print("bessel_i0.npz: %d values" % len(vals))


if __name__ == "__main__":
    main()
