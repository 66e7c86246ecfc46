"""Minimal PDB reading and writing for the command line: atom coordinates,
element, chain and atomic number (template weights), van der Waals radius
(molecular volume for the Fisher-z sigma) and rigid-body transforms of the
fitted copies.  Structure I/O is not part of the search; only what the
``powerfit`` command needs is here.
"""
from __future__ import annotations

import numpy as np

# atomic numbers and van der Waals radii (A, Bondi 1964) of the elements found
# in biomolecular models
ELEMENTS = {
    "H": (1, 1.20), "C": (6, 1.70), "N": (7, 1.55), "O": (8, 1.52), "F": (9, 1.47),
    "NA": (11, 2.27), "MG": (12, 1.73), "P": (15, 1.80), "S": (16, 1.80), "CL": (17, 1.75),
    "K": (19, 2.75), "CA": (20, 2.31), "MN": (25, 2.00), "FE": (26, 2.00), "CO": (27, 2.00),
    "NI": (28, 1.63), "CU": (29, 1.40), "ZN": (30, 1.39), "SE": (34, 1.90), "BR": (35, 1.85),
    "I": (53, 1.98),
}


class Structure:
    def __init__(self, records):
        self.records = records        # list of dicts (one per atom line)
        self.coor = np.array([[r["x"], r["y"], r["z"]] for r in records], dtype=np.float64).T.reshape(3, -1)

    @classmethod
    def fromfile(cls, fid):
        if hasattr(fid, "read"):
            text = fid.read()
        else:
            with open(fid) as f:
                text = f.read()
        recs = []
        for line in text.splitlines():
            if not line.startswith(("ATOM  ", "HETATM")):
                continue
            name = line[12:16]
            elem = line[76:78].strip().upper() if len(line) >= 78 else ""
            if not elem:
                elem = "".join(ch for ch in name if ch.isalpha())[:1].upper()
            recs.append(dict(line=line.ljust(80), x=float(line[30:38]), y=float(line[38:46]),
                             z=float(line[46:54]), chain=line[21], element=elem))
        return cls(recs)

    @property
    def data(self):
        return np.asarray(self.records)

    @property
    def atomnumber(self):
        return np.array([ELEMENTS.get(r["element"], (6, 1.7))[0] for r in self.records], dtype=np.float64)

    @property
    def rvdw(self):
        return np.array([ELEMENTS.get(r["element"], (6, 1.7))[1] for r in self.records], dtype=np.float64)

    def select(self, key, values):
        if key != "chain":
            raise ValueError("only chain selection is supported")
        values = set(values)
        return Structure([r for r in self.records if r["chain"] in values])

    def duplicate(self):
        s = Structure([dict(r) for r in self.records])
        s.coor = self.coor.copy()
        return s

    def translate(self, trans):
        self.coor += np.asarray(trans, dtype=np.float64).reshape(3, 1)

    def rotate(self, rotmat):
        self.coor = np.asarray(rotmat, dtype=np.float64) @ self.coor

    def tofile(self, fname):
        with open(fname, "w") as f:
            for r, (x, y, z) in zip(self.records, self.coor.T):
                line = r["line"]
                f.write(line[:30] + "%8.3f%8.3f%8.3f" % (x, y, z) + line[54:].rstrip() + "\n")
            f.write("END\n")


def write_fits_to_pdb(structure, solutions, basename="fit"):
    """One PDB per solution: centred structure, rotated, moved to the solution
    (reference ``helpers.py:54-64``)."""
    centred = structure.duplicate()
    centred.translate(-centred.coor.mean(axis=1))
    for n, sol in enumerate(solutions, start=1):
        out = centred.duplicate()
        out.rotate(np.asarray([float(v) for v in sol[6:]]).reshape(3, 3))
        out.translate(sol[3:6])
        out.tofile(basename + "_{:d}.pdb".format(n))
