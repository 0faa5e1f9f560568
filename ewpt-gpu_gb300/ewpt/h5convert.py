"""Convert the driver's NumPy outputs to the reference's HDF5 files.

    python -m ewpt.h5convert DIR

Writes DIR/data.h5 from DIR/data.npz and DIR/3d-fft-data-<it>.h5 from each
DIR/3d-fft-data-<it>.npz (ewpt.run), with the dataset names of
gpu-kernels-rk4/main_rk4.jl:6085-6092, 6861-6868 and 6930-6958.

The arrays in the .npz files carry the reference's Julia axes (A[x, y, z],
A[snap, column]).  HDF5.jl stores a Julia array with its dimensions reversed
(column-major memory, row-major dataspace), so each array is written here as
its transpose: a Julia reader (analysis-scripts/reader.jl) gets back the
original axes.  Complex arrays use h5py's compound {r, i}, the layout HDF5.jl
writes for Complex{Float64}.  Needs h5py, which is not part of this
project's dependencies.
"""
from __future__ import annotations

import glob
import os
import sys

import numpy as np


def julia_layout(a: np.ndarray) -> np.ndarray:
    """The row-major array whose dataspace HDF5.jl would write for the
    Julia-axes array a (dimensions reversed, same memory order)."""
    a = np.asarray(a)
    return np.ascontiguousarray(a.T) if a.ndim > 1 else a


def convert_file(src: str, dst: str) -> list:
    import h5py

    names = []
    with np.load(src) as z, h5py.File(dst, "w") as f:
        for k in z.files:
            f.create_dataset(k, data=julia_layout(z[k]))
            names.append(k)
    return names


def convert_dir(d: str) -> list:
    written = []
    for src in [os.path.join(d, "data.npz")] + sorted(glob.glob(os.path.join(d, "3d-fft-data-*.npz"))):
        if os.path.exists(src):
            dst = src[:-4] + ".h5"
            convert_file(src, dst)
            written.append(dst)
    return written


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print(__doc__)
        return 2
    try:
        import h5py  # noqa: F401
    except ImportError:
        print("h5py is not installed: the .npz files hold the same datasets", file=sys.stderr)
        return 1
    for w in convert_dir(argv[0]):
        print(w)
    return 0


if __name__ == "__main__":
    sys.exit(main())
