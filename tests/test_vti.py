"""The VTK dump (pfgpu_write_vti) without a GPU: the file is the one the
reference driver's writeVTK writes for the same arrays (gpuSEM_LB.c:1631-1709),
restated here in Python, byte for byte; downsampled fields carry their stride
in Spacing; bad arguments are refused on the host."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def gpu():
    from platelet_fiber_gpu_gb300 import build
    build.build()
    from platelet_fiber_gpu_gb300 import gpu as g
    return g


def reference_vti(nx, ny, nz, rho, ux, uy, uz, write_rho, write_vel, spacing=1):
    """gpuSEM_LB.c:1649-1708: header, Density then Velocity data arrays,
    "%.4e " per value, one line per x row ([z][y][x] order)."""
    out = ['<?xml version="1.0"?>\n', "<!-- gpuLBMflow ND ACMS -->\n",
           '<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n',
           '  <ImageData WholeExtent="0 %d 0 %d 0 %d" Origin="0 0 0" Spacing="%d %d %d">\n'
           % (nx - 1, ny - 1, nz - 1, spacing, spacing, spacing),
           '  <Piece Extent="0 %d 0 %d 0 %d">\n' % (nx - 1, ny - 1, nz - 1),
           '    <PointData Scalars="scalars">\n']
    if write_rho:
        out.append('      <DataArray type="Float32" Name="Density" NumberOfComponents="1" format="ascii">\n')
        for z in range(nz):
            for y in range(ny):
                out.append("".join("%.4e " % float(rho[z, y, x]) for x in range(nx)) + "\n")
        out.append("      </DataArray>\n")
    if write_vel:
        out.append('      <DataArray type="Float32" Name="Velocity" NumberOfComponents="3" format="ascii">\n')
        for z in range(nz):
            for y in range(ny):
                out.append("".join("%.4e %.4e %.4e " % (float(ux[z, y, x]), float(uy[z, y, x]), float(uz[z, y, x]))
                                   for x in range(nx)) + "\n")
        out.append("      </DataArray>\n")
    out += ["    </PointData>\n", "    <CellData>\n", "    </CellData>\n", "  </Piece>\n", "  </ImageData>\n",
            "</VTKFile>\n"]
    return "".join(out)


@pytest.mark.parametrize("write_rho,write_vel,spacing", [(1, 1, 1), (1, 0, 1), (0, 1, 2)])
def test_vti_matches_reference_writer(gpu, tmp_path, write_rho, write_vel, spacing):
    rng = np.random.default_rng(11)
    nz, ny, nx = 3, 4, 5
    rho = (1 + 1e-3 * rng.standard_normal((nz, ny, nx))).astype(np.float32)
    u = (1e-2 * rng.standard_normal((3, nz, ny, nx))).astype(np.float32)
    u[0, 0, 0, 0] = 0.0
    u[1, 0, 0, 1] = -0.0
    d = tmp_path / "Output"
    gpu.write_vti(42, rho, u, d, "LBMflow", spacing=spacing, write_rho=bool(write_rho), write_vel=bool(write_vel))
    got = (d / "LBMflow_0000042.vti").read_text()
    assert got == reference_vti(nx, ny, nz, rho, u[0], u[1], u[2], write_rho, write_vel, spacing)


def test_vti_refuses_bad_arguments(gpu, tmp_path):
    import ctypes as C
    L = gpu.lib()
    assert L.pfgpu_write_vti(0, 0, 1, 1, 1, None, 0, None, None, None, 0, str(tmp_path).encode(), b"x") == 1
    assert L.pfgpu_write_vti(0, 2, 2, 2, 1, None, 1, None, None, None, 0, str(tmp_path).encode(), b"x") == 1
    rho = np.ones(8, dtype=np.float32)
    p = rho.ctypes.data_as(C.POINTER(C.c_float))
    assert L.pfgpu_write_vti(0, 2, 2, 2, 0, p, 1, None, None, None, 0, str(tmp_path).encode(), b"x") == 1
    assert L.pfgpu_write_vti(0, 2, 2, 2, 1, p, 1, None, None, None, 0, str(tmp_path / "no" / "such").encode(),
                             b"x") == 1
