"""Reader for the reference's binary field file (``pglFieldStoreToFile``) for
kd-tree fields with (parallax-aware) VMMs at SIMD width 8
(PGL_DEVICE_TYPE_CPU_8) or 4, and with directional quadtrees (DQT.h:87-100,
DQTFactory.h:33-137: factory configuration, per region the quadtree nodes
and the statistics nodes).  Test infrastructure: it lets tests compare the reference's tree and
regions with the restatement in this folder and with the GPU library.

Layout (all little endian, packed as written by the stream writes):
  header string "OPENPGL_0.6.0_FIELD\\0", spatial type i32, directional type
  i32                                      (SurfaceVolumeField.h:197-214)
  iteration u64, totalSPP u64, surface Field, volume Field
                                           (SurfaceVolumeField.h:171-177)
  Field                                    (Field.h:240-267)
    isSurface b, decay f, iteration u64, totalSPP u64, deterministic b,
    fitRegions b, isSceneBoundsSet b, sceneBounds 6f, initialized b, 4 timings f
    factory config                         (AdaptiveSplitandMergeFactory.h:246-259,
                                            ParallaxAwareVonMisesFisherWeightedEMFactory.h:1335-1350)
    kd builder settings 3*u64              (KDTreeBuilder.h:377-382)
    kd tree: isInit b, bounds 6f, n u64, n * {split f, dimAndIdx u32}
                                           (KDTree.h:592-602, KDTree.h:136-140)
    regions u64, per region Region + Range (Region.h:63-71 of the survey's
                                            numbering: Region::serialize, Range.h)
    useStochasticNN b, KNN points          (KNN.h:320-331)
"""

from __future__ import annotations

import struct

import numpy as np

HEADER = b"OPENPGL_0.6.0_FIELD\x00"


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.o = 0

    def take(self, n):
        v = self.b[self.o : self.o + n]
        if len(v) != n:
            raise ValueError("field file truncated")
        self.o += n
        return v

    def u8(self):
        return self.take(1)[0]

    def i32(self):
        return struct.unpack("<i", self.take(4))[0]

    def u32(self):
        return struct.unpack("<I", self.take(4))[0]

    def u64(self):
        return struct.unpack("<Q", self.take(8))[0]

    def f32(self):
        return struct.unpack("<f", self.take(4))[0]

    def farr(self, n):
        return np.frombuffer(self.take(4 * n), dtype="<f4").copy()


def _lanes(r: _Reader, nvec, width, comps):
    """Reads nvec SIMD vectors of ``comps`` planes each; returns (comps, K)."""
    out = np.zeros((comps, nvec * width), dtype=np.float32)
    for k in range(nvec):
        for c in range(comps):
            out[c, k * width : (k + 1) * width] = r.farr(width)
    return out


def _read_field(r: _Reader, width: int, kmax: int = 32, dqt: bool = False):
    nvec = (kmax + width - 1) // width
    f = {}
    f["isSurface"] = bool(r.u8())
    f["decay"] = r.f32()
    f["iteration"] = r.u64()
    f["totalSPP"] = r.u64()
    f["deterministic"] = bool(r.u8())
    f["fitRegions"] = bool(r.u8())
    f["isSceneBoundsSet"] = bool(r.u8())
    f["_sceneBounds_offset"] = r.o
    f["sceneBounds"] = r.farr(6)
    f["initialized"] = bool(r.u8())
    f["_timings_offset"] = r.o
    f["timings"] = r.farr(4)
    if dqt:
        return _read_dqt_field(r, f)
    cfg = {}
    cfg["initK"] = r.u64()
    cfg["initKappa"] = r.f32()
    cfg["maxK"] = r.u64()
    cfg["maxEMIterations"] = r.u64()
    cfg["maxKappa"] = r.f32()
    cfg["maxMeanCosine"] = r.f32()
    cfg["convergenceThreshold"] = r.f32()
    cfg["weightPrior"] = r.f32()
    cfg["meanCosinePriorStrength"] = r.f32()
    cfg["meanCosinePrior"] = r.f32()
    cfg["splittingThreshold"] = r.f32()
    cfg["mergingThreshold"] = r.f32()
    cfg["partialReFit"] = bool(r.u8())
    cfg["maxSplitItr"] = r.i32()
    cfg["minSamplesForSplitting"] = r.i32()
    cfg["minSamplesForMerging"] = r.i32()
    cfg["minSamplesForPartialRefitting"] = r.i32()
    f["factory"] = cfg
    f["kd_settings"] = (r.u64(), r.u64(), r.u64())
    f["kd_isInit"] = bool(r.u8())
    f["_kd_bounds_offset"] = r.o
    f["kd_bounds"] = r.farr(6)
    nn = r.u64()
    raw = np.frombuffer(r.take(8 * nn), dtype=np.dtype([("split", "<f4"), ("bits", "<u4")])).copy()
    f["nodes"] = raw
    nreg = r.u64()
    regions = []
    for _ in range(nreg):
        g = {}
        g["valid"] = bool(r.u8())
        vm = {k: np.zeros(nvec * width, np.float32) for k in ("w", "kappa", "mx", "my", "mz", "norm", "e2k", "mc", "dist")}
        for k in range(nvec):
            sl = slice(k * width, (k + 1) * width)
            vm["w"][sl] = r.farr(width)
            vm["kappa"][sl] = r.farr(width)
            vm["mx"][sl] = r.farr(width)
            vm["my"][sl] = r.farr(width)
            vm["mz"][sl] = r.farr(width)
            vm["norm"][sl] = r.farr(width)
            vm["e2k"][sl] = r.farr(width)
            vm["mc"][sl] = r.farr(width)
            vm["dist"][sl] = r.farr(width)
        vm["K"] = r.u64()
        vm["pivot"] = r.farr(3)
        g["vmm"] = vm
        g["bounds"] = r.farr(6)
        ss = {k: np.zeros(nvec * width, np.float32) for k in ("dx", "dy", "dz", "w", "dw")}
        for k in range(nvec):
            sl = slice(k * width, (k + 1) * width)
            ss["dx"][sl] = r.farr(width)
            ss["dy"][sl] = r.farr(width)
            ss["dz"][sl] = r.farr(width)
            ss["w"][sl] = r.farr(width)
            ss["dw"][sl] = r.farr(width)
        ss["sumWeights"] = r.f32()
        ss["numSamples"] = r.f32()
        ss["overallNumSamples"] = r.f32()
        ss["K"] = r.u64()
        ss["normalized"] = bool(r.u8())
        g["suff"] = ss
        sp = {k: np.zeros(nvec * width, np.float32) for k in ("chi2", "mx", "my", "cx", "cy", "cz", "n", "sw", "sa")}
        for k in range(nvec):
            sl = slice(k * width, (k + 1) * width)
            sp["chi2"][sl] = r.farr(width)
            sp["mx"][sl] = r.farr(width)
            sp["my"][sl] = r.farr(width)
            sp["cx"][sl] = r.farr(width)
            sp["cy"][sl] = r.farr(width)
            sp["cz"][sl] = r.farr(width)
            sp["n"][sl] = r.farr(width)
            sp["sw"][sl] = r.farr(width)
            sp["sa"][sl] = r.farr(width)
        sp["K"] = r.u64()
        g["split"] = sp
        g["samplesAfterSplit"] = r.u64()
        g["samplesAfterMerge"] = r.u64()
        st = {}
        st["mean"] = r.farr(3)
        st["var"] = r.farr(3)
        st["n"] = r.f32()
        st["bounds"] = r.farr(6)
        g["stats"] = st
        g["splitFlag"] = bool(r.u8())
        g["range"] = (r.u64(), r.u64())
        regions.append(g)
    f["regions"] = regions
    f["useStochasticNN"] = bool(r.u8())
    built = bool(r.u8())
    f["knn_built"] = built
    if built:
        npnt = r.u32()
        f["knn_points"] = np.frombuffer(r.take(16 * npnt), dtype="<f4").reshape(npnt, 4)[:, :3].copy()
    return f


DQT_NODE = np.dtype([("offsetChildren", "<u4"), ("sampleWeight", "<f4")])
DQT_STATS_NODE = np.dtype([("offsetChildren", "<u4"), ("sampleWeight", "<f4"), ("splitWeight", "<f4"),
                           ("numSamples", "<f4"), ("firstMoment", "<f4"), ("secondMoment", "<f4")])


def _read_kd_and_tail(r: _Reader, f, read_region):
    f["kd_settings"] = (r.u64(), r.u64(), r.u64())
    f["kd_isInit"] = bool(r.u8())
    f["_kd_bounds_offset"] = r.o
    f["kd_bounds"] = r.farr(6)
    nn = r.u64()
    f["nodes"] = np.frombuffer(r.take(8 * nn), dtype=np.dtype([("split", "<f4"), ("bits", "<u4")])).copy()
    regions = []
    for _ in range(r.u64()):
        g = read_region(r)
        st = {}
        st["mean"] = r.farr(3)
        st["var"] = r.farr(3)
        st["n"] = r.f32()
        st["bounds"] = r.farr(6)
        g["stats"] = st
        g["splitFlag"] = bool(r.u8())
        g["range"] = (r.u64(), r.u64())
        regions.append(g)
    f["regions"] = regions
    f["useStochasticNN"] = bool(r.u8())
    built = bool(r.u8())
    f["knn_built"] = built
    if built:
        npnt = r.u32()
        f["knn_points"] = np.frombuffer(r.take(16 * npnt), dtype="<f4").reshape(npnt, 4)[:, :3].copy()
    return f


def _read_dqt_field(r: _Reader, f):
    # DirectionalQuadtreeFactory::Configuration, written as the raw struct
    f["factory"] = dict(leafEstimator=r.i32(), splitMetric=r.i32(), splitThreshold=r.f32(),
                        footprintFactor=r.f32(), maxLevels=r.u32())

    def region(r):
        g = {"valid": bool(r.u8())}
        pivot = r.farr(3)
        n = r.u64()
        g["dqt"] = {"pivot": pivot, "nodes": np.frombuffer(r.take(8 * n), dtype=DQT_NODE).copy()}
        g["bounds"] = r.farr(6)
        num = r.f32()
        n = r.u64()
        g["dqt_stats"] = {"numSamples": num, "nodes": np.frombuffer(r.take(24 * n), dtype=DQT_STATS_NODE).copy()}
        return g

    return _read_kd_and_tail(r, f, region)


def read_field_file(path_or_bytes, width: int = 8):
    buf = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    r = _Reader(bytes(buf))
    if r.take(len(HEADER)) != HEADER:
        raise ValueError("not an Open PGL 0.6.0 field file")
    out = {"spatialType": r.i32(), "directionalType": r.i32()}
    out["iteration"] = r.u64()
    out["totalSPP"] = r.u64()
    dqt = out["directionalType"] == 1  # PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE
    out["surface"] = _read_field(r, width, dqt=dqt)
    out["volume"] = _read_field(r, width, dqt=dqt)
    if r.o != len(r.b):
        raise ValueError(f"trailing bytes in field file: {len(r.b) - r.o}")
    return out


def node_is_leaf(bits):
    return (np.asarray(bits, np.uint32) >> 30) == 3


def canonical_tree(field):
    """Depth-first, left-first relabelling of nodes and leaves, as
    KDTree::rearrangeNodesForCompare (KDTree.h:256-283) does.  Returns
    (dims, split bits (u32), leaf flags, child index in canonical order,
    region index per canonical leaf)."""
    nodes = field["nodes"]
    if len(nodes) == 0:
        return dict(dim=np.zeros(0, np.int8), split=np.zeros(0, np.uint32), leaf=np.zeros(0, bool),
                    child=np.zeros(0, np.int64), region=np.zeros(0, np.int64))
    order = [0]
    canon_child = {}
    leaf_regions = []
    newpos = {0: 0}
    stack = [0]
    # iterative version of the recursive DFS: children appended as a pair,
    # then the left subtree fully before the right one
    out_nodes = [0]

    def visit(idx, new_idx):
        bits = int(nodes["bits"][idx])
        if (bits >> 30) != 3:
            left = bits & 0x3FFFFFFF
            base = len(out_nodes)
            canon_child[new_idx] = base
            out_nodes.append(left)
            out_nodes.append(left + 1)
            visit(left, base)
            visit(left + 1, base + 1)
        else:
            canon_child[new_idx] = len(leaf_regions)
            leaf_regions.append(bits & 0x3FFFFFFF)

    import sys

    sys.setrecursionlimit(10000)
    visit(0, 0)
    idx = np.array(out_nodes, dtype=np.int64)
    bits = nodes["bits"][idx]
    split = nodes["split"][idx].view(np.uint32)
    leaf = node_is_leaf(bits)
    dim = np.where(leaf, 3, bits >> 30).astype(np.int8)
    child = np.array([canon_child[i] for i in range(len(idx))], dtype=np.int64)
    return dict(dim=dim, split=np.where(leaf, 0, split).astype(np.uint32), leaf=leaf, child=child,
                region=np.array(leaf_regions, dtype=np.int64), split_f32=nodes["split"][idx])


def leaf_of_positions(field, pos):
    """Region index of each position by plain kd traversal (>= pivot goes
    right, KDTree.h:390-393)."""
    nodes = field["nodes"]
    pos = np.asarray(pos, np.float32)
    cur = np.zeros(len(pos), dtype=np.int64)
    bits = nodes["bits"].astype(np.int64)
    split = nodes["split"]
    active = (bits[cur] >> 30) != 3
    while active.any():
        b = bits[cur[active]]
        dim = b >> 30
        left = b & 0x3FFFFFFF
        p = pos[np.nonzero(active)[0], dim]
        cur[active] = left + (p >= split[cur[active]]).astype(np.int64)
        active = (bits[cur] >> 30) != 3
    return (bits[cur] & 0x3FFFFFFF).astype(np.int64)


def strip_timings(buf):
    """The field file with the bytes that do not describe the field set to
    zero, so that two files of the same field compare equal byte for byte:
    the per-field update timings (wall-clock values, Field.h:240-267) and, of
    a sub-field that was never initialised (no samples of its kind yet), the
    scene and kd-tree bounds, which the reference writes without having set
    them."""
    b = bytearray(buf)
    parsed = read_field_file(bytes(b))
    for side in ("surface", "volume"):
        f = parsed[side]
        o = f["_timings_offset"]
        b[o:o + 16] = bytes(16)
        if not f["initialized"]:
            for key in ("_sceneBounds_offset", "_kd_bounds_offset"):
                o = f[key]
                b[o:o + 24] = bytes(24)
    return bytes(b)
