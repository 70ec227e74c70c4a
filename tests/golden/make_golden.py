"""Regenerate the golden fixtures from the reference project's demo files.

The reference ships one known-answer case: demo/input.txt and the outputs its
GPU library wrote for it, demo/oname_w.txt (spectra) and demo/oname_t.txt
(time series).  This script copies the input and packs the defined part of the
outputs (columns 0-14 of a single-force run; columns 15-29 are zero there) into
tests/golden/demo_golden.npz.  It needs the reference checkout, so it runs only
where that is mounted, given as the argument or as GRTM_REFERENCE:

    python tests/golden/make_golden.py /path/to/reference
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_table(path, complex_pairs=False):
    rows = []
    with open(path) as f:
        for line in f:
            vals = [float(x) for x in line.strip().split(",") if x.strip()]
            if vals:
                rows.append(vals)
    a = np.array(rows)
    if complex_pairs:
        a = a[:, 0::2] + 1j * a[:, 1::2]
    return a


def main(ref):
    demo = os.path.join(ref, "demo")
    shutil.copyfile(os.path.join(demo, "input.txt"), os.path.join(HERE, "demo_input.txt"))
    shutil.copyfile(os.path.join(ref, "cusrc", "example", "crust1.0.txt"),
                    os.path.join(HERE, "example_crust1.0_input.txt"))
    w = read_table(os.path.join(demo, "oname_w.txt"), True)
    t = read_table(os.path.join(demo, "oname_t.txt"))
    n = w.shape[0]
    assert w.shape == (n, 30) and t.shape == (n, 30)
    np.savez_compressed(
        os.path.join(HERE, "demo_golden.npz"),
        spec=w[: n // 2 + 1, :15],           # rows above n/2 are conjugates (checked below)
        sig=t[:, :15],
        tail_max=np.array([np.abs(w[:, 15:]).max(), np.abs(t[:, 15:]).max()]),
        herm_err=np.array([np.abs(w[n // 2 + 1:, :] - np.conj(w[n // 2 - 1:0:-1, :])).max()]),
        nyquist_max=np.array([np.abs(w[n // 2, :]).max()]),
    )
    print("wrote", os.path.join(HERE, "demo_golden.npz"))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GRTM_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py REFERENCE_CHECKOUT (or set GRTM_REFERENCE)")
    main(ref)
