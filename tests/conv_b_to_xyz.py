"""Python 3 restatement of the reference's convBtoXYZ.py: splits a
cellsPos.data written as 32-bit floats (four per element: x, y, z, z) into
one XYZ file per frame, xyzFiles/pos_<frame>.xyz, each "<n>\\n   SCE\\n" then
"1 x y z" per element.  The original reads the file through `od -fv` and cuts
the address and the repeated z off every line; here the records are read
directly."""
from pathlib import Path

import numpy as np


def convert(data_file, n_sce: int, out_dir) -> int:
    rec = np.fromfile(data_file, dtype="<f4").reshape(-1, 4)
    frames = rec.shape[0] // n_sce
    out = Path(out_dir) / "xyzFiles"
    out.mkdir(parents=True, exist_ok=False)
    for i in range(frames):
        with open(out / f"pos_{i}.xyz", "w") as f:
            f.write(f"{n_sce}\n   SCE\n")
            for x, y, z, _ in rec[i * n_sce:(i + 1) * n_sce]:
                f.write(f"1 {x:.7e} {y:.7e} {z:.7e}\n")
    return frames


def read_xyz(path):
    lines = Path(path).read_text().splitlines()
    n = int(lines[0])
    return np.array([[float(v) for v in ln.split()[1:4]] for ln in lines[2:2 + n]])
