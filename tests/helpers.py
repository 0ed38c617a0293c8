"""Comparison helpers shared by the parity tests."""

import numpy as np

import fieldfile


def direction_grid(n=64):
    """Equal-area 64x64 grid of directions (z = 1 - 2u, phi = 2 pi v)."""
    u = (np.arange(n) + 0.5) / n
    z = 1.0 - 2.0 * u
    phi = 2.0 * np.pi * u
    zz, pp = np.meshgrid(z, phi, indexing="ij")
    r = np.sqrt(np.maximum(0.0, 1.0 - zz * zz))
    return np.stack([r * np.cos(pp), r * np.sin(pp), zz], axis=-1).reshape(-1, 3)


def vmm_pdf64(vmm, dirs):
    """Mixture pdf evaluated in FP64 from the stored lobe parameters."""
    K = int(vmm["K"])
    w = vmm["w"][:K].astype(np.float64)
    k = vmm["kappa"][:K].astype(np.float64)
    mu = np.stack([vmm["mx"][:K], vmm["my"][:K], vmm["mz"][:K]], axis=1).astype(np.float64)
    norm = np.where(k > 0, k / (2 * np.pi * (1 - np.exp(-2 * k))), 1 / (4 * np.pi))
    ct = dirs @ mu.T
    return (w * norm * np.exp(k * np.minimum(ct - 1.0, 0.0))).sum(axis=1)


def compare_fields(gpu_bytes, orc_bytes, side="surface", tol=1e-3):
    """Returns a dict describing how the GPU field matches the oracle field:
    tree and numbering equality, leaf sample statistics, regions whose
    mixture bytes are equal, the worst per-leaf relative PDF error on the
    64x64 grid, the leaves above `tol` (`over_tol`: region, error, lobe counts
    of both sides) and the leaves whose lobe count differs (`k_flips`: a split
    or merge decision that went the other way)."""
    A = fieldfile.read_field_file(gpu_bytes)[side]
    B = fieldfile.read_field_file(orc_bytes)[side]
    ca, cb = fieldfile.canonical_tree(A), fieldfile.canonical_tree(B)
    res = dict(tree_equal=bool(len(ca["dim"]) == len(cb["dim"]) and np.array_equal(ca["dim"], cb["dim"])
                               and np.array_equal(ca["split"], cb["split"])),
               numbering_equal=bool(len(A["nodes"]) == len(B["nodes"])
                                    and np.array_equal(A["nodes"]["bits"], B["nodes"]["bits"])),
               regions=len(A["regions"]))
    if not res["tree_equal"] or len(A["regions"]) != len(B["regions"]):
        return res
    dirs = direction_grid()
    bit = 0
    kdiff = 0
    worst = 0.0
    stats_equal = True
    rel_errs = []
    over, flips = [], []
    for ri, (ra, rb) in enumerate(zip(A["regions"], B["regions"])):
        for key in ("mean", "var", "bounds"):
            if not np.array_equal(ra["stats"][key].view(np.uint32), rb["stats"][key].view(np.uint32)):
                stats_equal = False
        if ra["stats"]["n"] != rb["stats"]["n"]:
            stats_equal = False
        va, vb = ra["vmm"], rb["vmm"]
        exact = va["K"] == vb["K"] and all(
            np.array_equal(va[k].view(np.uint32), vb[k].view(np.uint32))
            for k in ("w", "kappa", "mx", "my", "mz", "norm", "e2k", "mc", "dist"))
        bit += int(exact)
        if not (ra["valid"] and rb["valid"]):
            continue
        if va["K"] != vb["K"]:
            kdiff += 1
            flips.append((ri, int(va["K"]), int(vb["K"])))
        pa, pb = vmm_pdf64(va, dirs), vmm_pdf64(vb, dirs)
        rel = np.abs(pa - pb) / np.maximum(np.abs(pb), 1e-12)
        rel_errs.append(rel.max())
        worst = max(worst, float(rel.max()))
        if rel.max() > tol:
            over.append((ri, float(rel.max()), int(va["K"]), int(vb["K"])))
    res.update(bit_exact_regions=bit, k_differs=kdiff, worst_pdf_rel=worst, stats_equal=stats_equal,
               rel_errs=np.array(rel_errs), over_tol=over, k_flips=flips)
    return res


def compare_dqt_fields(a_bytes, b_bytes, side):
    """Two quadtree fields: kd-tree (canonical structure and node numbering),
    leaf sample statistics and pivots bit for bit, validity flags, and per
    region (in the fields' common numbering) the quadtree's child layout, the
    regions whose node and statistics bytes are equal, and the worst relative
    difference of node weights and training statistics."""
    A, B = fieldfile.read_field_file(a_bytes)[side], fieldfile.read_field_file(b_bytes)[side]
    ca, cb = fieldfile.canonical_tree(A), fieldfile.canonical_tree(B)
    res = dict(regions=len(A["regions"]), tree_equal=bool(np.array_equal(ca["dim"], cb["dim"])
                                                          and np.array_equal(ca["split"], cb["split"])),
               numbering_equal=bool(np.array_equal(A["nodes"]["bits"], B["nodes"]["bits"])))
    if not res["tree_equal"] or len(A["regions"]) != len(B["regions"]):
        return res
    worst, bit, structure, stats, valid = 0.0, 0, True, True, True
    for ra, rb in zip(A["regions"], B["regions"]):
        for key in ("mean", "var", "bounds"):
            if not np.array_equal(ra["stats"][key].view(np.uint32), rb["stats"][key].view(np.uint32)):
                stats = False
        if not np.array_equal(ra["dqt"]["pivot"].view(np.uint32), rb["dqt"]["pivot"].view(np.uint32)):
            stats = False
        valid &= ra["valid"] == rb["valid"]
        na, nb = ra["dqt"]["nodes"], rb["dqt"]["nodes"]
        if len(na) != len(nb) or not np.array_equal(na["offsetChildren"], nb["offsetChildren"]):
            structure = False
            continue
        sa, sb = ra["dqt_stats"]["nodes"], rb["dqt_stats"]["nodes"]
        same = na.tobytes() == nb.tobytes() and sa.tobytes() == sb.tobytes()
        bit += int(same)
        for x, y in ((na["sampleWeight"], nb["sampleWeight"]), (sa["sampleWeight"], sb["sampleWeight"]),
                     (sa["splitWeight"], sb["splitWeight"]), (sa["numSamples"], sb["numSamples"]),
                     (sa["firstMoment"], sb["firstMoment"]), (sa["secondMoment"], sb["secondMoment"])):
            x, y = x.astype(np.float64), y.astype(np.float64)
            rel = np.abs(x - y) / np.maximum(np.abs(y), 1e-30)
            worst = max(worst, float(rel.max()) if len(rel) else 0.0)
    res.update(structure_equal=structure, stats_equal=stats, valid_equal=bool(valid), bit_exact_regions=bit,
               worst_rel=worst)
    return res


def summary(r):
    """The comparison without the per-leaf error array (for messages and
    bench lines)."""
    return {k: v for k, v in r.items() if k != "rel_errs"}


def compare_queries(out, ref):
    """Guided-query agreement: same ok flags, region ids and rescaled sample1D
    bits; worst relative pdf error and direction difference over valid
    queries."""
    ok = ref["ok"] == 1
    res = dict(ok_equal=bool(np.array_equal(out["ok"], ref["ok"])),
               id_equal=bool(np.array_equal(out["id"][ok], ref["id"][ok])),
               sample1d_equal=bool(np.array_equal(out["sample1d"][ok].view(np.uint32),
                                                  ref["sample1d"][ok].view(np.uint32))),
               valid=int(ok.sum()))
    if ok.any():
        rel = np.abs(out["pdf"][ok].astype(np.float64) - ref["pdf"][ok]) / ref["pdf"][ok]
        res["worst_pdf_rel"] = float(rel.max())
        res["worst_dir"] = float(np.abs(out["dir"][ok] - ref["dir"][ok]).max())
        res["pdf_bit_exact_frac"] = float(np.mean(out["pdf"][ok].view(np.uint32) == ref["pdf"][ok].view(np.uint32)))
    else:
        res.update(worst_pdf_rel=0.0, worst_dir=0.0, pdf_bit_exact_frac=1.0)
    return res


def leaf_log_likelihoods(field_bytes, samples, side="surface"):
    """Per region: the weighted log-likelihood sum_i w_i log pdf(d_i) of the
    region's samples under its mixture, in FP64, with the samples reprojected
    onto the region's mean as the parallax-aware fit sees them
    (WEMFactory.h:1151-1196: distance max(9 sqrt(|variance|), d)).  Meant for
    the first Update of a field, where a region's sample statistics are those
    of the samples given.  Returns {region: (LL, sum_i w_i |log pdf(d_i)|)},
    the second a scale for relative comparisons (LL itself can be near 0)."""
    f = fieldfile.read_field_file(field_bytes)[side]
    pos = np.stack([samples["position"][:, i] for i in range(3)], axis=1).astype(np.float64)
    d = np.stack([samples["direction"][:, i] for i in range(3)], axis=1).astype(np.float64)
    w = samples["weight"].astype(np.float64)
    dist = samples["distance"].astype(np.float64)
    leaf = fieldfile.leaf_of_positions(f, pos.astype(np.float32))
    out = {}
    for r, reg in enumerate(f["regions"]):
        m = leaf == r
        if not m.any() or not reg["valid"]:
            continue
        st = reg["stats"]
        mean = st["mean"].astype(np.float64)
        var = st["var"].astype(np.float64) / float(st["n"])
        min_d = 9.0 * np.sqrt(np.sqrt((var * var).sum()))
        p, dd, ww, di = pos[m], d[m].copy(), w[m], dist[m]
        ok = np.isfinite(di) & (di > 0.0)
        dm = np.maximum(min_d, di[ok])
        o = p[ok] + dd[ok] * dm[:, None]
        nd = o - mean
        dd[ok] = nd / np.sqrt((nd * nd).sum(axis=1))[:, None]
        v = reg["vmm"]
        K = int(v["K"])
        mu = np.stack([v["mx"][:K], v["my"][:K], v["mz"][:K]], axis=1).astype(np.float64)
        kap, nrm, wk = (v[k][:K].astype(np.float64) for k in ("kappa", "norm", "w"))
        pdf = (wk[None, :] * nrm[None, :] * np.exp(kap[None, :] * (dd @ mu.T - 1.0))).sum(axis=1)
        good = pdf > 0
        t = ww[good] * np.log(pdf[good])
        out[r] = (float(t.sum()), float(np.abs(t).sum()))
    return out


def poisoned_frames():
    """Two frames; the second carries samples with NaN directions, NaN
    weights, infinite distances and zero weights."""
    from openpgl_gb300 import synthetic as syn

    frames = [syn.cube_face_samples(20000, 991 + i, volume_fraction=0.3) for i in range(2)]
    f = frames[1].copy()
    idx = np.random.default_rng(5).choice(len(f), 12, replace=False)
    f["direction"][idx[:3]] = np.nan
    f["weight"][idx[3:6]] = np.nan
    f["distance"][idx[6:9]] = np.inf
    f["weight"][idx[9:12]] = 0.0
    frames[1] = f
    return frames
