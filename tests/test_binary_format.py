"""OpenFOAM binary files (writeFormat binary, as in the reference's 3D
example, examples/3D_Cylinder_Re3900/S/system/controlDict:57): a binary
polyMesh (points, faceCompactList faces, owner, neighbour) and binary initial
fields read into the same solver description as the ASCII case, and the
driver's binary output equals its ASCII output bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases
from tests.helpers import load_golden, rel_l2

_MESHES = {
    "o-grid": lambda: cases.cylinder_case(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=1, minmod=True,
                                          noise=0.02),
    "3d-cyclic": lambda: cases.cylinder_case(n_theta=16, n_r=8, n_span=4, r1=6, first=0.05, Ls=2, noise=0.01),
    "triangles": lambda: cases.tri_case(n=8, seed=3),
    "tetrahedra": lambda: cases.tet_case(n=3, nz=2, seed=2),
}


def _arrays(ch):
    d = ch.desc
    out = {}
    for name, n in (("S", d.dim * d.n_faces), ("d", d.dim * d.n_faces), ("w", d.n_faces), ("K", d.dim * d.n_faces),
                    ("vol_inv", d.n_cells), ("sponge", d.n_cells), ("q0", d.nq * d.n_cells)):
        out[name] = ch.array(name, (n,))
    out["face_n"] = ch.array("face_n", (d.n_faces,), np.int64)
    return out


@pytest.mark.parametrize("name", sorted(_MESHES))
def test_binary_case_reads_like_ascii(tmp_path, name):
    c = _MESHES[name]()
    cases.write_case(c, str(tmp_path / "a"), n_steps=3)
    cases.write_case(c, str(tmp_path / "b"), n_steps=3, binary=True)
    head = open(tmp_path / "b" / "constant" / "polyMesh" / "faces", "rb").read(600)
    assert b"binary" in head and b"faceCompactList" in head
    a = _arrays(N.CaseHandle.open(str(tmp_path / "a")))
    b = _arrays(N.CaseHandle.open(str(tmp_path / "b")))
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_binary_field_reader_round_trip(tmp_path):
    c = _MESHES["o-grid"]()
    d = tmp_path / "0"
    d.mkdir()
    cases.write_field(c, str(d), "p", c.fields["p"], "[1 -1 -2 0 0 0 0]", binary=True)
    cases.write_field(c, str(d), "U", c.fields["U"], "[0 1 -1 0 0 0 0]", binary=True)
    assert np.array_equal(cases._read_internal_field(str(d / "p")), c.fields["p"])
    assert np.array_equal(cases._read_internal_field(str(d / "U")), c.fields["U"])


@pytest.mark.gpu
def test_driver_binary_run_equals_ascii_run(tmp_path):
    """lfm_solve_gpu on the binary case writes binary fields equal to the
    ASCII run's (17 significant digits: every double round-trips), both
    within 1e-12 of the reference's own run of the case."""
    cli = os.path.join(os.path.dirname(N.LIB_PATH), "lfm_solve_gpu")
    if not os.path.exists(cli):
        pytest.fail(f"{cli} is missing: build() makes it")
    case, z = load_golden("cyl24x12_m2")
    n = int(z["n_steps"])
    out = {}
    for fmt in ("ascii", "binary"):
        root = str(tmp_path / fmt)
        cases.write_case(case, root, n_steps=n, binary=(fmt == "binary"))
        r = subprocess.run([cli], cwd=root, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        out[fmt] = cases.read_result_fields(root)
        tdirs = [x for x in os.listdir(root) if x not in ("0", "constant", "system", "output")]
        head = open(os.path.join(root, max(tdirs, key=float), "p"), "rb").read(400)
        assert (b"binary" in head) == (fmt == "binary")
    for k in ("rho", "E", "p", "U"):
        assert np.array_equal(out["ascii"][k], out["binary"][k]), k
    for k in ("rho", "E", "p"):
        assert rel_l2(out["binary"][k][None], z["ref_" + k][None])[0] <= 1e-12, k
    shutil.rmtree(str(tmp_path), ignore_errors=True)
