"""SOLUTION.OUT writer (write_solution layout): edit descriptors and record shapes."""
from __future__ import annotations

import numpy as np

from movfem_gb300 import output


def test_edit_descriptors():
    assert output.es(1.0) == "         1.00000E+00"
    assert output.es(-2.5e-7) == "        -2.50000E-07"
    assert output.es(0.0) == "         0.00000E+00"
    assert output.es(6.02214076e123) == "         6.02214+123"
    assert output.fw(12.345678) == "            12.34568"
    assert output.fw(-0.5) == "            -0.50000"
    assert len(output.es(1.0)) == 20 and len(output.fw(1.0)) == 20


def test_block_layout_and_round_trip():
    rng = np.random.Generator(np.random.PCG64(3))
    npt = 5
    E = rng.normal(size=(npt, 2, 3)) + 1j * rng.normal(size=(npt, 2, 3))
    H = rng.normal(size=(npt, 2, 3)) + 1j * rng.normal(size=(npt, 2, 3))
    Z = rng.normal(size=(npt, 4)) + 1j * rng.normal(size=(npt, 4))
    rho = rng.uniform(0, 100, size=(npt, 4))
    phi = rng.uniform(-90, 90, size=(npt, 4))
    lines = output.solution_block(2, E, H, Z, rho, phi).splitlines()
    assert lines[0] == " vector-fem solution:            2"
    assert len(lines) == 1 + (1 + npt) * 3
    assert len(lines[1]) == 24 * 15 and lines[1].startswith("     Re[Ex_(1)]")
    rec = lines[2]
    assert len(rec) == 24 * 20
    vals = [float(rec[20 * i:20 * i + 20]) for i in range(24)]
    ref = []
    for p in range(2):
        ref += [v for a in range(3) for v in (E[0, p, a].real, E[0, p, a].imag)]
        ref += [v for a in range(3) for v in (H[0, p, a].real, H[0, p, a].imag)]
    np.testing.assert_allclose(vals, ref, rtol=1e-5, atol=1e-5)
    zrec = lines[2 + npt + 1]
    assert len(zrec) == 8 * 20
    rrec = lines[-1]
    np.testing.assert_allclose([float(rrec[20 * i:20 * i + 20]) for i in range(8)],
                               list(rho[-1]) + list(phi[-1]), atol=1e-5)


def test_receiver_file_layout(tmp_path):
    rng = np.random.Generator(np.random.PCG64(4))
    nf, nrx = 2, 3
    rx = rng.uniform(0, 1000, size=(nrx, 2))
    E = rng.normal(size=(nf, nrx, 2, 3)) + 1j * rng.normal(size=(nf, nrx, 2, 3))
    H = rng.normal(size=(nf, nrx, 2, 3)) + 1j * rng.normal(size=(nf, nrx, 2, 3))
    Z = rng.normal(size=(nf, nrx, 4)) + 1j * rng.normal(size=(nf, nrx, 4))
    rho = rng.uniform(0, 10, size=(nf, nrx, 4))
    phi = rng.uniform(-90, 90, size=(nf, nrx, 4))
    path = tmp_path / "RECEIVER.OUT"
    output.write_receivers(str(path), rx, np.zeros(nrx), E, H, Z, rho, phi)
    lines = path.read_text().splitlines()
    assert len(lines) == 2 + nrx + nf * 3 * (1 + nrx)
    head = lines[2 + nrx]
    assert head.startswith("    1 ") and len(head) == 6 + 26 * 15
    rec = lines[3 + nrx]
    assert len(rec) == 26 * 20
    assert abs(float(rec[:20]) - rx[0, 0]) < 1e-3 * max(1.0, abs(rx[0, 0]))
    assert abs(float(rec[40:60]) - E[0, 0, 0, 0].real) < 1e-5 * max(1.0, abs(E[0, 0, 0, 0].real))
    assert lines[-1 - nrx].startswith("    2 ") and len(lines[-1]) == 10 * 20


def test_surface_file_layout(tmp_path):
    from movfem_gb300 import mesh as M
    m = M.layered_blocks(3, nodes_per_elem=8, ncx=4, ncy=3, ncz=2, d=100.0, nextd=1, n_air=2, dz_air=100.0,
                         nfreq=2, fmin=1.0, fmax=10.0, nrx=2)
    ids = output.surface_nodes(m)
    # inner grid without the extension cells, at the earth surface
    assert ids.size == (m.nnx - 2) * (m.nny - 2)
    assert np.allclose(np.asarray(m.zp)[ids], m.ztop)
    rng = np.random.Generator(np.random.PCG64(5))
    nf, npt = 2, m.npt
    E = rng.normal(size=(nf, npt, 2, 3)) + 0j
    H = rng.normal(size=(nf, npt, 2, 3)) + 0j
    Z = rng.normal(size=(nf, npt, 4)) + 0j
    rho = rng.uniform(0, 10, size=(nf, npt, 4))
    phi = rng.uniform(-90, 90, size=(nf, npt, 4))
    path = tmp_path / "SURFACE.OUT"
    output.write_surface(str(path), m, E, H, Z, rho, phi)
    lines = path.read_text().splitlines()
    assert len(lines) == 5 + nf * 3 * (1 + ids.size)
    rec = lines[6]
    assert abs(float(rec[:20]) - E[0, ids[0], 0, 0].real) < 1e-5 * max(1.0, abs(E[0, ids[0], 0, 0].real))
