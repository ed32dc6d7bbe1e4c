"""Element dumps in the reference driver's formats (pfgpu_output_*):
cellsPos.data records (x, RY, z, z) per element per frame, the initial-only
velocity and force records, the ASCII tables, the pause-time record, and the
float mode read back through the convBtoXYZ.py restatement."""
import numpy as np
import pytest

from conv_b_to_xyz import convert, read_xyz

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def _positions(E):
    return np.stack([E["X"], E["RY"], E["Z"], E["Z"]], axis=1)


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_output_frames(gpu, tmp_path, fp32):
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    PE = sc.n_platelets * sc.n_elem
    j = gpu.Job(sc, 1)
    E0 = j.elements()
    out = j.output(tmp_path, fp32=fp32)
    frames = [E0]
    for _ in range(2):
        j.step(3)
        out.frame()
        frames.append(j.elements())
    out.close(seed=11)
    dt = np.float32 if fp32 else np.float64
    pos = np.fromfile(tmp_path / "cellsPos.data", dtype=dt).reshape(-1, 4)
    assert pos.shape[0] == 3 * PE
    for k, E in enumerate(frames):
        np.testing.assert_array_equal(pos[k * PE:(k + 1) * PE], _positions(E).astype(dt))
    vel = np.fromfile(tmp_path / "cellsVel.data", dtype=dt).reshape(-1, 4)
    force = np.fromfile(tmp_path / "cellsForce.data", dtype=dt).reshape(-1, 4)
    assert vel.shape[0] == force.shape[0] == PE  # initial frame only
    V, F = E0["V"], E0["F"]
    np.testing.assert_array_equal(vel[:, :3], V.T.astype(dt))
    np.testing.assert_array_equal(force[:, 2], F[2].astype(dt))
    table = (tmp_path / "cellsPosASCII.dat").read_text().split("\n")
    assert table[0].split() == ["Timestep", "ElemID", "X", "Y", "Z"]
    rows = [r.split() for r in table[1:] if r.strip()]
    assert len(rows) == 3 * PE
    assert rows[0][:2] == ["0", "0"] and rows[PE][:2] == ["3", "0"] and rows[-1][:2] == ["6", str(sc.n_elem - 1)]
    np.testing.assert_allclose([float(v) for v in rows[-1][2:]], _positions(frames[-1])[-1, :3], rtol=1e-6)
    pause = (tmp_path / "cellsPauseTime.dat").read_text().strip().split(",")
    assert int(pause[1]) == 11
    assert float(pause[0]) == pytest.approx(6 * float(np.float32(sc.dt)), rel=1e-6)
    j.close()
    if fp32:
        n = convert(tmp_path / "cellsPos.data", PE, tmp_path)
        assert n == 3
        xyz = read_xyz(tmp_path / "xyzFiles" / "pos_2.xyz")
        np.testing.assert_allclose(xyz, _positions(frames[2])[:, :3], rtol=1e-6)


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "fp32", "fp16"])
def test_fields_and_vti(gpu, tmp_path, prec):
    """pfgpu_job_get_fields (density and velocity computed on the device at
    every stride-th node) agrees with the full lattice download rounded to
    float, before the first step and after some; stride 2 is the subsample of
    stride 1; the job's VTK dump holds those values at "%.4e"."""
    import xml.etree.ElementTree as ET
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    j = gpu.Job(sc, prec)
    for steps in (0, 5):
        j.step(steps)
        full = j.lattice(fIN=False)
        shape = (sc.nz, sc.ny, sc.nx)
        f1 = j.fields(1)
        np.testing.assert_array_equal(f1["rho"], full["rho"].reshape(shape).astype(np.float32))
        np.testing.assert_array_equal(f1["u"], full["u"].reshape((3,) + shape).astype(np.float32))
        f2 = j.fields(2)
        np.testing.assert_array_equal(f2["rho"], f1["rho"][::2, ::2, ::2])
        np.testing.assert_array_equal(f2["u"], f1["u"][:, ::2, ::2, ::2])
    j.write_vti(5, tmp_path / "Output", stride=2)
    root = ET.parse(tmp_path / "Output" / "LBMflow_0000005.vti").getroot()
    img = root.find("ImageData")
    mz, my, mx = f2["rho"].shape
    assert img.get("WholeExtent") == "0 %d 0 %d 0 %d" % (mx - 1, my - 1, mz - 1)
    assert img.get("Spacing") == "2 2 2"
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=np.float64) for a in img.iter("DataArray")}
    np.testing.assert_allclose(arrays["Density"], f2["rho"].ravel(), rtol=6e-5)
    vel = np.stack([f2["u"][i].ravel() for i in range(3)], axis=1).ravel()
    np.testing.assert_allclose(arrays["Velocity"], vel, rtol=6e-5, atol=1e-30)
    j.close()
