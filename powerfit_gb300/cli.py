"""``powerfit``-compatible command line on the GB300 search.

Same arguments and flow as the reference CLI (``powerfit.py:25-319``):
read the map, resample to ``--resampling-rate`` x Nyquist, trim, extend to a
2,3,5,7-smooth shape, read the structure, build template and mask (on the
GPU), pick the rotation set, optional core weighting, scan, analyse, write
``lcc.mrc``, ``solutions.out`` and ``fit_N.pdb``.

``-g/--gpu`` is accepted for compatibility (the search always runs on the
GPU); ``-p/--nproc`` is accepted and ignored.  ``--device`` picks the CUDA
device.  Rotation sets are the reference's Karney files, read from
``--rotation-data`` or ``$POWERFIT_ROTATION_DATA``; without them a
super-Fibonacci set of the same size is used and the log says so.
"""
from __future__ import annotations

import logging
import os
import sys
from argparse import ArgumentParser, FileType
from time import time

import numpy as np


def parse_args(argv=None):
    p = ArgumentParser(prog="powerfit")
    p.add_argument("target", type=FileType("rb"), help="Target density map (CCP4 or MRC).")
    p.add_argument("resolution", type=float, help="Resolution of map in angstrom")
    p.add_argument("template", type=FileType("r"), help="Atomic model to be fitted (PDB).")
    p.add_argument("-a", "--angle", dest="angle", type=float, default=10, metavar="<float>")
    p.add_argument("-l", "--laplace", dest="laplace", action="store_true")
    p.add_argument("-cw", "--core-weighted", dest="core_weighted", action="store_true")
    p.add_argument("-nr", "--no-resampling", dest="no_resampling", action="store_true")
    p.add_argument("-rr", "--resampling-rate", dest="resampling_rate", type=float, default=2, metavar="<float>")
    p.add_argument("-nt", "--no-trimming", dest="no_trimming", action="store_true")
    p.add_argument("-tc", "--trimming-cutoff", dest="trimming_cutoff", type=float, default=None, metavar="<float>")
    p.add_argument("-c", "--chain", dest="chain", type=str, default=None, metavar="<char>")
    p.add_argument("-d", "--directory", dest="directory", type=os.path.abspath, default=".", metavar="<dir>")
    p.add_argument("-n", "--num", dest="num", type=int, default=10, metavar="<int>")
    p.add_argument("-g", "--gpu", dest="gpu", action="store_true")
    p.add_argument("-p", "--nproc", dest="nproc", type=int, default=1, metavar="<int>")
    p.add_argument("--device", dest="device", type=int, default=0, metavar="<int>")
    p.add_argument("--rotation-data", dest="rotation_data", default=None, metavar="<dir>")
    return p.parse_args(argv)


def fisher_sigma(mv, fsc):
    return 1 / np.sqrt(mv / fsc - 3)


def main(argv=None):
    t0 = time()
    args = parse_args(argv)
    os.makedirs(args.directory, exist_ok=True)
    log = logging.getLogger("powerfit_gb300.cli")
    log.setLevel(logging.INFO)
    handler = logging.FileHandler(os.path.join(args.directory, "powerfit.log"))
    handler.setFormatter(logging.Formatter("%(asctime)s %(message)s"))
    log.addHandler(handler)

    def write(line):
        if sys.stdout.isatty():
            print(line)
        log.info(line)

    try:
        return _run(args, write, t0)
    finally:
        log.removeHandler(handler)
        handler.close()


def _run(args, write, t0):
    from . import CUDACorrelator
    from .analyzer import Analyzer
    from ._lib import core_indices
    from .rotations import rotation_set
    from .structure import Structure, write_fits_to_pdb
    from .volume import Volume, extend, nearest_multiple2357, resample, structure_to_shape_like, trim

    write(" ".join(sys.argv))
    target = Volume.fromfile(args.target)
    write("Target resolution: {:.2f}".format(args.resolution))
    if not args.no_resampling:
        factor = 2 * args.resampling_rate * target.voxelspacing / args.resolution
        if factor < 0.9:
            target = resample(target, factor)
    if not args.no_trimming:
        cutoff = args.trimming_cutoff if args.trimming_cutoff is not None else target.array.max() / 10
        target = trim(target, cutoff)
    target = extend(target, [nearest_multiple2357(n) for n in target.shape])
    write(("Shape after extending:" + " {:d}" * 3).format(*target.shape))

    structure = Structure.fromfile(args.template)
    if args.chain is not None:
        structure = structure.select("chain", args.chain.split(","))
    if structure.coor.shape[1] == 0:
        raise ValueError("No atoms were selected.")
    structure.translate(np.asarray(target.origin, dtype=np.float64) - structure.coor.mean(axis=1))
    template = structure_to_shape_like(target, structure.coor, resolution=args.resolution,
                                       weights=structure.atomnumber, shape="vol")
    mask = structure_to_shape_like(target, structure.coor, resolution=args.resolution, shape="mask")

    rotmat, desc = rotation_set(args.angle, data_dir=args.rotation_data)
    write("Rotation set: " + desc)
    if args.core_weighted:
        mask.array = core_indices(mask.array)         # on the GPU

    corr = CUDACorrelator(target.array, laplace=args.laplace, device=args.device)
    corr.template = template.array
    corr.mask = mask.array
    corr.rotations = rotmat
    t1 = time()
    corr.scan()
    write("Time for search: {:.0f}m {:.0f}s".format(*divmod(time() - t1, 60)))

    mv = structure_to_shape_like(target, structure.coor, resolution=args.resolution, radii=structure.rvdw,
                                 shape="mask").array.sum() * target.voxelspacing ** 3
    analyzer = Analyzer(corr.lcc, rotmat, corr.rot, voxelspacing=target.voxelspacing, origin=target.origin,
                        z_sigma=fisher_sigma(mv, args.resolution))
    Volume(corr.lcc, target.voxelspacing, target.origin).tofile(os.path.join(args.directory, "lcc.mrc"))
    analyzer.tofile(os.path.join(args.directory, "solutions.out"))
    n = min(args.num, len(analyzer.solutions))
    write_fits_to_pdb(structure, analyzer.solutions[:n], basename=os.path.join(args.directory, "fit"))
    write("Total time: {:.0f}m {:.0f}s".format(*divmod(time() - t0, 60)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
