"""End-to-end ``powerfit`` command on a small synthetic map (GPU)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write_pdb(path, coords, elements):
    names = {6: "C", 7: "N", 8: "O", 16: "S"}
    with open(path, "w") as f:
        for i, ((x, y, z), e) in enumerate(zip(coords, elements), start=1):
            el = names[int(e)]
            f.write("ATOM  %5d  %-3s ALA A%4d    %8.3f%8.3f%8.3f  1.00  0.00          %2s\n"
                    % (i, el, i, x, y, z, el))


def test_powerfit_cli_finds_the_planted_copy(tmp_path):
    from powerfit_gb300 import synth
    from powerfit_gb300.cli import main
    from powerfit_gb300.volume import Volume, read_map
    c = synth.make_case((48, 48, 48), 2.5, 400, 1, 8.0, 10.0, seed=17)
    mp = str(tmp_path / "target.mrc")
    Volume(c.target.astype(np.float64), 2.5, (0.0, 0.0, 0.0)).tofile(mp)
    # the copy in the map is chain @ R^T + centre; give the CLI the unrotated chain
    pdb = str(tmp_path / "model.pdb")
    _write_pdb(pdb, c.chain + 40.0, c.elements)
    out = str(tmp_path / "out")
    rc = main([mp, "8.0", pdb, "-a", "20", "-nr", "-nt", "-d", out, "-n", "3"])
    assert rc == 0
    for f in ("lcc.mrc", "solutions.out", "fit_1.pdb", "powerfit.log"):
        assert os.path.exists(os.path.join(out, f)), f
    lcc, vs, _ = read_map(os.path.join(out, "lcc.mrc"))
    assert lcc.shape == (48, 48, 48) and lcc.max() > 0.3
    best = open(os.path.join(out, "solutions.out")).read().splitlines()[1].split()
    pos = np.array([float(best[4]), float(best[5]), float(best[6])])
    assert np.linalg.norm(pos - c.copy_centres[0]) < 3 * 2.5
