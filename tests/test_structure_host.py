"""PDB reading and writing of the command line (CPU only): atom records,
element inference, template weights, chain selection, rigid transforms and
the per-solution fit files (reference helpers.py:54-64: centre the
structure, rotate it, move it to the solution)."""
import numpy as np

from powerfit_gb300.structure import Structure, write_fits_to_pdb

PDB = """\
HEADER    TEST
ATOM      1  N   ALA A   1      11.104   6.134  -6.504  1.00  0.00           N
ATOM      2  CA  ALA A   1      11.639   6.071  -5.147  1.00  0.00           C
ATOM      3  O   ALA A   1      12.000   7.000  -4.000  1.00  0.00
HETATM    4 FE   HEM B   2       1.000   2.000   3.000  1.00  0.00          FE
ATOM      5  SG  CYS B   3      -1.500   0.250   4.750  1.00  0.00           S
TER
END
"""


def _structure(tmp_path):
    path = tmp_path / "in.pdb"
    path.write_text(PDB)
    return Structure.fromfile(str(path))


def test_reads_atoms_elements_and_weights(tmp_path):
    s = _structure(tmp_path)
    assert s.coor.shape == (3, 5)
    assert np.allclose(s.coor[:, 0], [11.104, 6.134, -6.504])
    assert [r["element"] for r in s.records] == ["N", "C", "O", "FE", "S"]   # O from the atom name
    assert [r["chain"] for r in s.records] == ["A", "A", "A", "B", "B"]
    assert np.array_equal(s.atomnumber, [7, 6, 8, 26, 16])
    assert np.allclose(s.rvdw, [1.55, 1.70, 1.52, 2.00, 1.80])
    with open(tmp_path / "in.pdb") as f:                           # an open file works too
        assert Structure.fromfile(f).coor.shape == (3, 5)


def test_select_duplicate_and_transforms(tmp_path):
    s = _structure(tmp_path)
    b = s.select("chain", ["B"])
    assert b.coor.shape == (3, 2) and np.allclose(b.coor[:, 0], [1, 2, 3])
    d = s.duplicate()
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], dtype=np.float64)
    d.rotate(R)
    d.translate([1, 2, 3])
    assert np.allclose(d.coor, R @ s.coor + np.array([[1], [2], [3]]))
    assert np.allclose(s.coor[:, 0], [11.104, 6.134, -6.504])     # the original is untouched


def test_tofile_round_trip(tmp_path):
    s = _structure(tmp_path)
    s.translate([0.5, -0.25, 1.0])
    out = tmp_path / "out.pdb"
    s.tofile(str(out))
    t = Structure.fromfile(str(out))
    assert np.allclose(t.coor, s.coor, atol=5e-4)
    assert [r["element"] for r in t.records] == [r["element"] for r in s.records]
    assert out.read_text().rstrip().endswith("END")


def test_fit_files_centre_rotate_and_place(tmp_path):
    s = _structure(tmp_path)
    R = np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], dtype=np.float64)
    pos = np.array([10.0, 20.0, 30.0])
    sol = np.concatenate([[0.9, 1.47, 5.0], pos, R.ravel()])       # (lcc, Fisher z, relative z, x, y, z, rotation)
    write_fits_to_pdb(s, [sol], basename=str(tmp_path / "fit"))
    fit = Structure.fromfile(str(tmp_path / "fit_1.pdb"))
    centred = s.coor - s.coor.mean(axis=1, keepdims=True)
    assert np.allclose(fit.coor, R @ centred + pos[:, None], atol=5e-4)
