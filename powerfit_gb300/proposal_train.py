"""Train the proposal network on seeded synthetic maps and measure it on held-out seeds.

Every training pair comes from the exhaustive search itself: for each map,
the coarse search's per-rotation best LCC gives the features and the
full-resolution search's per-rotation best LCC gives the target.  Validation
maps (at the held-out grid size) pick the training variant and, for the
network and for the coarse score alone, the operating fraction: the smallest
re-searched fraction at which the ranking keeps its best fits (stored with
the weights).  The held-out maps are searched three ways -- exhaustively,
with the network's proposal and with the coarse score alone (the method
without the network), each at its own operating fraction -- and the script
reports best-fit recall and time to best fit.  The seeded maps are built in
worker processes while the GPU searches.

    python -m powerfit_gb300.proposal_train --maps 200 --valid 24 --eval 100 --workers 12 \\
        --out powerfit_gb300/data/proposal_net.npz --report powerfit_gb300/data/proposal_net_report.json
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

from . import proposal as PR
from . import synth

SET_SIZE = 207576            # the 3.26 deg set (the reference's c48u8649 size): the "3 deg" set
TRAIN_SEED0 = 1000
VALID_SEED0 = 800000         # validation seeds: pick the training variant
EVAL_SEED0 = 900000          # held-out seeds never used for training or selection
VARIANTS = ("all", "candidates")


def case_params(seed, edge):
    """Seeded map parameters: 1,000-8,000 atoms, 5-9 A, SNR 1-6, 1-3 copies, a
    voxel spacing that leaves the chain inside the rotation sphere."""
    rng = np.random.default_rng(seed)
    natoms = int(rng.integers(1000, 8001))
    res = float(rng.uniform(5.0, 9.0))
    snr = float(rng.uniform(1.0, 6.0))
    ncopies = int(rng.integers(1, 4))
    rg = 25.0 * (natoms / 4000.0) ** (1.0 / 3.0)
    vs = float(np.clip(2.2 * 2.0 * 1.4 * rg * (1.0 + 0.35 * (ncopies - 1)) / edge, 1.2, 3.0))
    return dict(natoms=natoms, resolution=res, snr=snr, ncopies=ncopies, voxelspacing=vs)


def synth_case(job):
    """The seeded map of (seed, edge): its parameters and the arrays a
    SearchPair takes (run in worker processes while the GPU searches)."""
    seed, edge = job
    prm = case_params(seed, edge)
    case = synth.make_case((edge,) * 3, prm["voxelspacing"], prm["natoms"], prm["ncopies"], prm["resolution"],
                           prm["snr"], seed)
    return dict(seed=seed, params=prm, target=case.target, template=case.template, mask=case.mask,
                voxelspacing=case.voxelspacing, resolution=case.resolution)


def _cases(seeds, edge, pool=None):
    """The maps of `seeds` in order, built on `pool` (a spawn-started process
    pool) ahead of their use, or here one by one."""
    jobs = [(s, edge) for s in seeds]
    return pool.imap(synth_case, jobs) if pool is not None else map(synth_case, jobs)


def pair_of(d, rotmats, device=0):
    return PR.SearchPair(d["target"], d["template"], d["mask"], d["voxelspacing"], d["resolution"], rotmats,
                         laplace=False, core_weighted=False, device=device)


def make_pair(seed, edge, rotmats, device=0):
    d = synth_case((seed, edge))
    return pair_of(d, rotmats, device), d["params"]


def search_data(seeds, edge, rotmats, device=0, log=print, pool=None):
    """Per map: the coarse search's per-rotation (best LCC, voxel), the coarse
    grid, and the full-resolution per-rotation best LCC (the exhaustive search)."""
    out = []
    t0 = time.perf_counter()
    for i, d in enumerate(_cases(seeds, edge, pool)):
        pair = pair_of(d, rotmats, device)
        coarse = pair.coarse_scores()
        _, _, fine = pair.fine_exhaustive(rotation_max=True)
        out.append(dict(seed=d["seed"], coarse=coarse, shape=pair.coarse.shape, fine=fine))
        pair.close()
        log("map %d/%d seed %d %s: %.1f s" % (i + 1, len(seeds), d["seed"], d["params"], time.perf_counter() - t0))
        t0 = time.perf_counter()
    return out


def build(maps, nbr, variant, device=0):
    """Training tensors (x, t, w) of one variant:
    ``all``: every rotation, the top 5% (by full-resolution score) weighted 10x;
    ``candidates``: only the coarse top 20% of each map (the ranking that
    matters), its top 1% weighted 10x."""
    import torch
    xs, ts, ws = [], [], []
    for m in maps:
        x = PR.features(m["coarse"], nbr, m["shape"], device)
        t, w = PR.targets(m["fine"], device)
        if variant == "candidates":
            cs = torch.as_tensor(np.nan_to_num(m["coarse"][0], nan=-np.inf), device=x.device)
            keep = cs >= torch.quantile(cs[torch.isfinite(cs)], 0.8)
            x, t = x[keep], t[keep]
            w = 1.0 + 9.0 * (t >= torch.quantile(t, 0.99)).float()
        xs.append(x)
        ts.append(t)
        ws.append(w)
    return torch.cat(xs).contiguous(), torch.cat(ts).contiguous(), torch.cat(ws).contiguous()


def best_rank(score, fine, tol):
    """Rank of the best-fit rotation (any within `tol` of the best LCC) under `score`."""
    f = np.nan_to_num(np.asarray(fine, dtype=np.float64), nan=-np.inf)
    good = f >= f.max() - tol
    return int(np.min(np.sum(score[None, :] > score[good][:, None], axis=1)))


def rank_quality(net, maps, nbr, device=0):
    """Mean log10 rank fraction of the best rotation over validation maps."""
    vals = []
    for m in maps:
        score = PR.rank_scores(net, m["coarse"], nbr, m["shape"], device).float().cpu().numpy()
        r = best_rank(score, m["fine"], FOUND_TOL) / float(score.size)
        vals.append(math.log10(r + 1e-6))
    return float(np.mean(vals)), vals


# Two searches that score the same rotation agree to about 1e-7 (a rotation's
# partner in the packed complex transform changes the rounding), so the best
# fit counts as found within this LCC tolerance.
FOUND_TOL = 1e-5
FRACTIONS = (0.05, 0.02, 0.01, 0.005)
# Operating fraction of a ranking, chosen on validation maps: the smallest of
# CANDIDATE_FRACTIONS at which at least SELECT_RECALL of the maps rank their
# best fit inside the fraction divided by SELECT_MARGIN (a margin for maps
# that validation has not seen).
CANDIDATE_FRACTIONS = (0.002, 0.005, 0.01, 0.02, 0.05, 0.1)
SELECT_RECALL = 0.99
SELECT_MARGIN = 2.0


def choose_fraction(ranks, nrot):
    """Operating fraction of a ranking from its validation ranks (see above); 1.0
    (the exhaustive search) if no candidate keeps the recall."""
    ranks = np.asarray(ranks, dtype=np.float64)
    for f in CANDIDATE_FRACTIONS:
        if np.mean(ranks < f * nrot / SELECT_MARGIN) >= SELECT_RECALL:
            return f
    return 1.0


def validation_ranks(net, maps, nbr, device=0):
    """Rank of each map's best fit under the network (or the coarse score, `net` None)."""
    out = []
    for m in maps:
        score = PR.rank_scores(net, m["coarse"], nbr, m["shape"], device).float().cpu().numpy()
        out.append(best_rank(score, m["fine"], FOUND_TOL))
    return out


def evaluate(net, seeds, edge, rotmats, nbr, device=0, fractions=None, log=print, pool=None):
    """Per held-out map: exhaustive time and best fit; for the network and for
    the coarse score alone, each at its operating fraction (``fractions``:
    {"network": f, "coarse_only": f}, default TOP_FRACTION for both): whether
    the best fit was found, the rank of the best rotation (recall at other
    fractions follows from it), time to best fit."""
    import torch
    fractions = fractions or {"network": PR.TOP_FRACTION, "coarse_only": PR.TOP_FRACTION}
    rows = []
    for d in _cases(seeds, edge, pool):
        seed, prm = d["seed"], d["params"]
        pair = pair_of(d, rotmats, device)
        # warm both searches and the ranking (first launches, autotuned shapes) outside the timings
        c0 = pair.coarse_scores()
        for model in (net, None):
            PR.select(PR.rank_scores(model, c0, nbr, pair.coarse.shape, device))
        pair.fine_subset(np.arange(min(512, pair.nrot)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lcc_x, rot_x, fine = pair.fine_exhaustive(rotation_max=True)
        torch.cuda.synchronize()
        t_ex = time.perf_counter() - t0
        best = float(lcc_x.max())
        best_rot = int(np.argmax(np.nan_to_num(fine, nan=-np.inf)))
        row = dict(seed=seed, params=prm, exhaustive_s=t_ex, best_lcc=best, best_rotation=best_rot)
        s = pair.coarse_scores()
        for name, model in (("network", net), ("coarse_only", None)):
            score = PR.rank_scores(model, s, nbr, pair.coarse.shape, device).float().cpu().numpy()
            timings = {}
            frac = fractions[name]
            lcc_p, rot_p, sel = PR.proposal_search(pair, model, nbr, frac, timings)
            found = float(lcc_p.max()) >= best - FOUND_TOL
            # a rotation scoring within the tolerance of the best counts as the best fit too
            rank = best_rank(score, fine, FOUND_TOL)
            row[name] = dict(found=bool(found), rank=rank, rank_fraction=rank / pair.nrot, fraction=frac,
                             found_at={str(f): bool(rank < math.ceil(f * pair.nrot)) for f in FRACTIONS},
                             best_lcc=float(lcc_p.max()), time_s=timings["total_s"], timings=timings)
        pair.close()
        log(json.dumps(row))
        rows.append(row)
    return rows


def summarise(rows):
    out = {}
    for name in ("network", "coarse_only"):
        out[name] = dict(
            recall=float(np.mean([r[name]["found"] for r in rows])),
            recall_at={str(f): float(np.mean([r[name]["found_at"][str(f)] for r in rows])) for f in FRACTIONS},
            median_rank_fraction=float(np.median([r[name]["rank_fraction"] for r in rows])),
            worst_rank_fraction=float(np.max([r[name]["rank_fraction"] for r in rows])),
            time_s=float(np.mean([r[name]["time_s"] for r in rows])),
            fraction=rows[0][name].get("fraction"),
        )
    ex = float(np.mean([r["exhaustive_s"] for r in rows]))
    out["exhaustive_s"] = ex
    for name in ("network", "coarse_only"):
        out[name]["time_vs_exhaustive"] = out[name]["time_s"] / ex
    return out


def operating_fractions(path):
    """The operating fractions stored with trained weights ({"network": f,
    "coarse_only": f}), or TOP_FRACTION for both where the file has none."""
    import ast
    with np.load(path) as d:
        meta = ast.literal_eval(str(d["meta"])) if "meta" in d.files else {}
    fr = meta.get("fractions") if isinstance(meta, dict) else None
    return dict(fr) if fr else {"network": PR.TOP_FRACTION, "coarse_only": PR.TOP_FRACTION}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--maps", type=int, default=64, help="training maps")
    ap.add_argument("--valid", type=int, default=24, help="validation maps (variant and operating fractions)")
    ap.add_argument("--edge", type=int, default=96, help="training grid edge")
    ap.add_argument("--valid-edge", type=int, default=128, help="validation grid edge")
    ap.add_argument("--eval", type=int, default=12, help="held-out maps")
    ap.add_argument("--eval-edge", type=int, default=128)
    ap.add_argument("--set-size", type=int, default=SET_SIZE)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--workers", type=int, default=8, help="processes building the seeded maps")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                                  "proposal_net.npz"))
    ap.add_argument("--report", default=None, help="write the evaluation summary (JSON) here")
    ap.add_argument("--weights", default=None, help="evaluate these weights instead of training")
    args = ap.parse_args(argv)
    import multiprocessing as mp
    pool = mp.get_context("spawn").Pool(max(1, args.workers)) if args.workers > 0 else None
    import torch
    from .rotations import quat_to_rotmat, super_fibonacci
    torch.cuda.set_device(0)
    log = lambda m: print(m, flush=True)
    rotmats = quat_to_rotmat(super_fibonacci(args.set_size))
    t0 = time.perf_counter()
    nbr = PR.rotation_neighbours(rotmats)
    log("neighbour table %.1f s" % (time.perf_counter() - t0))
    choice = {}
    if args.weights:
        net = PR.ProposalNet.load(args.weights)
        fractions = operating_fractions(args.weights)
        history = []
    else:
        seeds = [TRAIN_SEED0 + i for i in range(args.maps)]
        train = search_data(seeds, args.edge, rotmats, log=log, pool=pool)
        valid = search_data([VALID_SEED0 + i for i in range(args.valid)], args.valid_edge, rotmats, log=log,
                            pool=pool)
        base_q, _ = rank_quality(None, valid, nbr)
        choice["coarse_only"] = base_q
        best = None
        for variant in VARIANTS:
            x, t, w = build(train, nbr, variant)
            cand = PR.ProposalNet(seed=0)
            t1 = time.perf_counter()
            hist = cand.train(x, t, w, epochs=args.epochs, lr=args.lr, log=log)
            torch.cuda.synchronize()
            q, per_map = rank_quality(cand, valid, nbr)
            choice[variant] = q
            log("variant %s: %d samples, %.1f s, validation mean log10 rank %.3f (coarse only %.3f) %s"
                % (variant, x.shape[0], time.perf_counter() - t1, q, base_q, [round(v, 2) for v in per_map]))
            if best is None or q < best[0]:
                best = (q, variant, cand, hist)
            del x, t, w
        _, variant, net, history = best
        # operating fractions of the kept network and of the coarse score alone, on the validation maps
        ranks = {"network": validation_ranks(net, valid, nbr), "coarse_only": validation_ranks(None, valid, nbr)}
        fractions = {k: choose_fraction(v, rotmats.shape[0]) for k, v in ranks.items()}
        log("validation ranks %s -> operating fractions %s" % (ranks, fractions))
        os.makedirs(os.path.dirname(args.out), exist_ok=True)
        net.save(args.out, meta=dict(maps=args.maps, edge=args.edge, set_size=args.set_size, epochs=args.epochs,
                                     lr=args.lr, seeds=[seeds[0], seeds[-1]], variant=variant,
                                     validation=choice, final_loss=history[-1], fractions=fractions,
                                     validation_ranks=ranks, valid_maps=args.valid, valid_edge=args.valid_edge))
    rows = evaluate(net, [EVAL_SEED0 + i for i in range(args.eval)], args.eval_edge, rotmats, nbr,
                    fractions=fractions, log=log, pool=pool)
    if pool is not None:
        pool.close()
    summary = summarise(rows)
    summary.update(train_loss=history[-3:] if history else None, validation=choice, set_size=args.set_size,
                   fractions=fractions, eval_edge=args.eval_edge, eval_maps=args.eval)
    log(json.dumps(summary))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(dict(summary=summary, rows=rows), f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
