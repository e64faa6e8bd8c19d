"""Extract the reference's historic golden trajectories into small .npy fixtures.

The reference's examples/*.py scripts run 1000-2000 quasistatic steps and
compare (x_frame | u_frame, f_frame, S) with the stored .h5 files.  h5py is not
available here, so this script reads the HDF5 files' raw bytes: each file holds
three contiguous little-endian datasets of n 8-byte values, stored one after
the other from byte 2048 in creation order.  The dataset names are asserted in
the object header before the data are read.

Run from the repository root:  python tests/golden/make_golden.py <reference-root>
"""

import pathlib
import sys

import numpy as np

FILES = {
    "Line1d_Cuspy_Laplace": (1000, "x_frame"),
    "Line2d_Cuspy_Laplace": (1000, "x_frame"),
    "Line1d_SemiSmooth_Laplace": (1000, "x_frame"),
    "Particles_Cuspy": (2000, "u_frame"),
    "Line1d_Cuspy_Laplace_Nopassing": (1000, "x_frame"),
    "Line1d_Cuspy_Quartic": (1000, "x_frame"),
    "Line1d_Cuspy_Laplace_LongRange": (200, "x_frame"),
}
# third dataset "t_insta" (float) instead of "S" (int)
THERMAL = {"Line1d_System_Cuspy_Laplace_RandomForcing": 500}


def read(path: pathlib.Path, n: int, first: str):
    raw = path.read_bytes()
    header = raw[:2048]
    for name in (first, "f_frame", "S"):
        assert (name + "\x00").encode() in header, (path, name)
    assert len(raw) == 2048 + 3 * 8 * n, (path, len(raw))
    frame = np.frombuffer(raw[2048 : 2048 + 8 * n], "<f8").copy()
    f_frame = np.frombuffer(raw[2048 + 8 * n : 2048 + 16 * n], "<f8").copy()
    S = np.frombuffer(raw[2048 + 16 * n : 2048 + 24 * n], "<i8").copy()
    return frame, f_frame, S


def main():
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {pathlib.Path(__file__).name} <root of the reference project>")
    ref = pathlib.Path(sys.argv[1])
    out = pathlib.Path(__file__).parent
    for stem, (n, first) in FILES.items():
        frame, f_frame, S = read(ref / "examples" / (stem + ".h5"), n, first)
        np.savez(out / (stem + ".npz"), frame=frame, f_frame=f_frame, S=S)
        print(stem, frame[-1], f_frame[-1], S.sum())
    for stem, n in THERMAL.items():
        raw = (ref / "examples" / (stem + ".h5")).read_bytes()
        for name in ("x_frame", "f_frame", "t_insta"):
            assert (name + "\x00").encode() in raw[:2048], (stem, name)
        assert len(raw) == 2048 + 3 * 8 * n, (stem, len(raw))
        cols = [np.frombuffer(raw[2048 + 8 * n * i: 2048 + 8 * n * (i + 1)], "<f8").copy() for i in range(3)]
        np.savez(out / (stem + ".npz"), frame=cols[0], f_frame=cols[1], t_insta=cols[2])
        print(stem, cols[0][-1], cols[1][-1], cols[2][-1])


if __name__ == "__main__":
    main()
