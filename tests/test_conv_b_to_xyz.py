"""The convBtoXYZ.py restatement on a synthetic float record file."""
import numpy as np

from conv_b_to_xyz import convert, read_xyz


def test_frames_split_and_values(tmp_path):
    rng = np.random.default_rng(1)
    n, frames = 7, 3
    pos = rng.normal(size=(frames, n, 3)).astype(np.float32)
    rec = np.concatenate([pos, pos[..., 2:3]], axis=-1)
    rec.astype("<f4").tofile(tmp_path / "cellsPos.data")
    assert convert(tmp_path / "cellsPos.data", n, tmp_path) == frames
    for i in range(frames):
        xyz = read_xyz(tmp_path / "xyzFiles" / f"pos_{i}.xyz")
        np.testing.assert_allclose(xyz, pos[i], rtol=1e-6)
    head = (tmp_path / "xyzFiles" / "pos_0.xyz").read_text().splitlines()[:2]
    assert head == [str(n), "   SCE"]
