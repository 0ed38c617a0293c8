"""Seeded synthetic sample and query generators for the field-training and
guided-query workloads (the shapes the Open PGL benchmark tool feeds to
``Field::Update`` and to the sampling distributions; the reference ships no
sample files, so these stand in for them).

Every value is produced from PCG64 uniforms using only correctly rounded
IEEE operations (+, -, *, /, sqrt, floor, comparisons, sorting).  No libm
transcendental is called, because exp/log/sin differ in the last bit between
libm builds and CPU architectures; exp and log below are deterministic series
built from the basic operations.  The same seed therefore gives bit-identical
samples on any machine, which lets golden outputs produced on one host be
checked on another.

Record layout: ``PGL_SAMPLE_DTYPE`` is the 40-byte ``PGLSampleData``
(openpgl/include/openpgl/data.h:21-49): position f3, direction f3, weight,
pdf, distance (f32) and flags (u32; bit 1 = inside volume).
"""

from __future__ import annotations

import numpy as np

PGL_SAMPLE_DTYPE = np.dtype(
    [
        ("position", "<f4", (3,)),
        ("direction", "<f4", (3,)),
        ("weight", "<f4"),
        ("pdf", "<f4"),
        ("distance", "<f4"),
        ("flags", "<u4"),
    ]
)
assert PGL_SAMPLE_DTYPE.itemsize == 40

# Guided query record: position, normal, sample1D, two uniforms (36 bytes).
PGL_QUERY_DTYPE = np.dtype(
    [("position", "<f4", (3,)), ("normal", "<f4", (3,)), ("sample1d", "<f4"), ("u", "<f4", (2,))]
)
assert PGL_QUERY_DTYPE.itemsize == 36

# Path vertex with four 2D random numbers (PGLGuidedVertex, 76 bytes).
PGL_VERTEX_DTYPE = np.dtype(
    [("position", "<f4", (3,)), ("normal", "<f4", (3,)), ("wo", "<f4", (3,)), ("roughness", "<f4"),
     ("sample1d", "<f4"), ("u", "<f4", (4, 2))]
)
assert PGL_VERTEX_DTYPE.itemsize == 76

FLAG_INSIDE_VOLUME = 2
_LN2 = 0.6931471805599453
_INV_4PI = 0.07957747154594767


def det_exp(x):
    """exp(x) as (1 + x/2^20)^(2^20) by 20 squarings (basic ops only)."""
    y = 1.0 + np.asarray(x, dtype=np.float64) / 1048576.0
    for _ in range(20):
        y = y * y
    return y


def det_log(x):
    """log(x) for x > 0: exact binary exponent plus an atanh series."""
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)  # exact: x = m * 2^e, m in [0.5, 1)
    z = (m - 1.0) / (m + 1.0)
    z2 = z * z
    s = np.zeros_like(z)
    for k in range(29, 0, -2):  # z * sum z^(2j) / (2j+1)
        s = s * z2 + 1.0 / k
    return 2.0 * z * s + e * _LN2


def _normal(rng, shape):
    """Approximately standard normal: Irwin-Hall sum of 12 uniforms - 6."""
    acc = np.zeros(shape, dtype=np.float64)
    for _ in range(12):
        acc += rng.random(shape)
    return acc - 6.0


def _unit_sphere(rng, n):
    """Uniform directions by rejection from the cube (deterministic rounds)."""
    out = np.empty((0, 3), dtype=np.float64)
    while out.shape[0] < n:
        m = max(64, 2 * (n - out.shape[0]) + 64)
        c = rng.random((m, 3)) * 2.0 - 1.0
        r2 = (c * c).sum(axis=1)
        keep = (r2 > 1e-6) & (r2 <= 1.0)
        c = c[keep] / np.sqrt(r2[keep])[:, None]
        out = np.concatenate([out, c])
    return out[:n]


def _lobe_directions(rng, mu, kappa):
    """vMF-like lobe: normalize(mu + g / sqrt(kappa)), g ~ N(0, I)."""
    g = _normal(rng, mu.shape)
    d = mu + g / np.sqrt(kappa)[:, None]
    return d / np.sqrt((d * d).sum(axis=1))[:, None]


def _dirichlet1(rng, n, k):
    """Dirichlet(1,...,1) weights as spacings of sorted uniforms."""
    u = np.sort(rng.random((n, k - 1)), axis=1)
    edges = np.concatenate([np.zeros((n, 1)), u, np.ones((n, 1))], axis=1)
    return np.diff(edges, axis=1)


def _pick(rng, weights):
    """Index drawn from each row of a weight matrix (inverse CDF)."""
    cdf = np.cumsum(weights, axis=1)
    u = rng.random(weights.shape[0]) * cdf[:, -1]
    return np.minimum((cdf < u[:, None]).sum(axis=1), weights.shape[1] - 1)


def _pack(pos, d, w, pdf, dist, flags):
    s = np.zeros(pos.shape[0], dtype=PGL_SAMPLE_DTYPE)
    s["position"] = pos.astype(np.float32)
    s["direction"] = d.astype(np.float32)
    s["weight"] = w.astype(np.float32)
    s["pdf"] = pdf.astype(np.float32)
    s["distance"] = dist.astype(np.float32)
    s["flags"] = flags.astype(np.uint32)
    return s


def cube_face_samples(n, seed, volume_fraction=0.0):
    """Surface samples uniform on the 6 faces of [0,1]^3 with directions from
    a 3-lobe mixture chosen per position octant (lobe means uniform on the
    sphere, kappa log-uniform in [5, 200], Dirichlet(1) lobe weights),
    lognormal(0,1) weights, pdf 1/(4 pi), distance U[0.05, 2].

    With ``volume_fraction`` > 0 that share of the samples carries the
    inside-volume flag, sits uniformly in the cube interior and takes its
    direction from one lobe with kappa = 20 (one lobe mean per seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lobe_mu = _unit_sphere(rng, 8 * 3).reshape(8, 3, 3)
    lobe_kappa = 5.0 * det_exp(rng.random((8, 3)) * det_log(40.0))
    lobe_w = _dirichlet1(rng, 8, 3)
    vol_mu = _unit_sphere(rng, 1)[0]

    face = np.minimum(np.floor(rng.random(n) * 6.0), 5.0).astype(np.int64)
    uv = rng.random((n, 2))
    pos = np.empty((n, 3), dtype=np.float64)
    axis = face % 3
    side = (face // 3).astype(np.float64)
    for a in range(3):
        sel = axis == a
        o1, o2 = (a + 1) % 3, (a + 2) % 3
        pos[sel, a] = side[sel]
        pos[sel, o1] = uv[sel, 0]
        pos[sel, o2] = uv[sel, 1]
    is_vol = rng.random(n) < volume_fraction
    pos[is_vol] = rng.random((int(is_vol.sum()), 3))
    octant = ((pos[:, 0] >= 0.5) * 4 + (pos[:, 1] >= 0.5) * 2 + (pos[:, 2] >= 0.5)).astype(np.int64)
    lobe = _pick(rng, lobe_w[octant])
    mu = lobe_mu[octant, lobe]
    kappa = lobe_kappa[octant, lobe]
    mu[is_vol] = vol_mu
    kappa = np.where(is_vol, 20.0, kappa)
    d = _lobe_directions(rng, mu, kappa)
    w = det_exp(_normal(rng, n))
    dist = 0.05 + 1.95 * rng.random(n)
    pdf = np.full(n, _INV_4PI)
    flags = np.where(is_vol, FLAG_INSIDE_VOLUME, 0)
    return _pack(pos, d, w, pdf, dist, flags)


def cluster_model(seed, num_clusters=4096):
    """4096 isotropic Gaussian clusters: centres uniform in [0,1]^3, sigma
    log-uniform in [1e-3, 5e-2], Zipf(1.1) masses, 1-6 lobes per cluster with
    kappa log-uniform in [2, 1000] and Dirichlet(1) weights."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centers = rng.random((num_clusters, 3))
    sigma = 1e-3 * det_exp(rng.random(num_clusters) * det_log(50.0))
    ranks = np.arange(1, num_clusters + 1, dtype=np.float64)
    mass = det_exp(-1.1 * det_log(ranks))
    rng.shuffle(mass)
    nlobes = 1 + np.minimum(np.floor(rng.random(num_clusters) * 6.0), 5.0).astype(np.int64)
    mu = _unit_sphere(rng, num_clusters * 6).reshape(num_clusters, 6, 3)
    kappa = 2.0 * det_exp(rng.random((num_clusters, 6)) * det_log(500.0))
    w = _dirichlet1(rng, num_clusters, 6)
    w[np.arange(6)[None, :] >= nlobes[:, None]] = 0.0
    return dict(centers=centers, sigma=sigma, mass=mass / mass.sum(), mu=mu, kappa=kappa, lobe_w=w)


def cluster_samples(n, seed, model_seed=1234, volume_fraction=0.0, num_clusters=4096):
    """Samples around the clusters of ``cluster_model``; lognormal(0,2)
    weights (heavy tailed), pdf 1/(4 pi), distance U[0.05, 2]."""
    m = cluster_model(model_seed, num_clusters)
    rng = np.random.Generator(np.random.PCG64(seed))
    cdf = np.cumsum(m["mass"])
    c = np.minimum(np.searchsorted(cdf, rng.random(n) * cdf[-1], side="right"), num_clusters - 1)
    pos = m["centers"][c] + m["sigma"][c][:, None] * _normal(rng, (n, 3))
    lobe = _pick(rng, m["lobe_w"][c])
    d = _lobe_directions(rng, m["mu"][c, lobe], m["kappa"][c, lobe])
    w = det_exp(2.0 * _normal(rng, n))
    dist = 0.05 + 1.95 * rng.random(n)
    pdf = np.full(n, _INV_4PI)
    is_vol = rng.random(n) < volume_fraction
    flags = np.where(is_vol, FLAG_INSIDE_VOLUME, 0)
    return _pack(pos, d, w, pdf, dist, flags)


def queries(n, seed, model_seed=None, num_clusters=4096):
    """Guided queries: position uniform in [0,1]^3 (or drawn from the cluster
    model when ``model_seed`` is given), normal uniform on the sphere,
    sample1D and u uniform in [0,1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    q = np.zeros(n, dtype=PGL_QUERY_DTYPE)
    if model_seed is None:
        pos = rng.random((n, 3))
    else:
        m = cluster_model(model_seed, num_clusters)
        cdf = np.cumsum(m["mass"])
        c = np.minimum(np.searchsorted(cdf, rng.random(n) * cdf[-1], side="right"), num_clusters - 1)
        pos = m["centers"][c] + m["sigma"][c][:, None] * _normal(rng, (n, 3))
    q["position"] = pos.astype(np.float32)
    q["normal"] = _unit_sphere(rng, n).astype(np.float32)
    # float32 values strictly below 1 (the reference asserts sample1D < 1)
    q["sample1d"] = np.minimum(rng.random(n), 0.99999994).astype(np.float32)
    q["u"] = np.minimum(rng.random((n, 2)), 0.99999994).astype(np.float32)
    return q


def vertices(n, seed, model_seed=1234, num_clusters=4096):
    """Path vertices of the serving workload: position drawn from the cluster
    model, normal and outgoing direction uniform on the sphere, roughness,
    sample1D and four 2D random numbers uniform in [0,1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = np.zeros(n, dtype=PGL_VERTEX_DTYPE)
    m = cluster_model(model_seed, num_clusters)
    cdf = np.cumsum(m["mass"])
    c = np.minimum(np.searchsorted(cdf, rng.random(n) * cdf[-1], side="right"), num_clusters - 1)
    v["position"] = (m["centers"][c] + m["sigma"][c][:, None] * _normal(rng, (n, 3))).astype(np.float32)
    v["normal"] = _unit_sphere(rng, n).astype(np.float32)
    v["wo"] = _unit_sphere(rng, n).astype(np.float32)
    v["roughness"] = rng.random(n).astype(np.float32)
    v["sample1d"] = np.minimum(rng.random(n), 0.99999994).astype(np.float32)
    v["u"] = np.minimum(rng.random((n, 4, 2)), 0.99999994).astype(np.float32)
    return v


def vertex_queries(v, k):
    """The single-sample guided queries equal to SamplePDF call k of each
    vertex (same position, normal and sample1D, the k-th 2D random number)."""
    q = np.zeros(len(v), dtype=PGL_QUERY_DTYPE)
    q["position"] = v["position"]
    q["normal"] = v["normal"]
    q["sample1d"] = v["sample1d"]
    q["u"] = v["u"][:, k]
    return q


def frames_blob(frames):
    """Serialise a list of sample arrays as u64 count + (u64 n + records)*."""
    parts = [np.uint64(len(frames)).tobytes()]
    for f in frames:
        parts.append(np.uint64(len(f)).tobytes())
        parts.append(np.ascontiguousarray(f).tobytes())
    return b"".join(parts)


def queries_blob(q):
    return np.uint64(len(q)).tobytes() + np.ascontiguousarray(q).tobytes()


# PGLPathSegmentData (data.h), 136 bytes
PGL_PATH_SEGMENT_DTYPE = np.dtype(
    [("position", "<f4", (3,)), ("direction_in", "<f4", (3,)), ("direction_out", "<f4", (3,)),
     ("normal", "<f4", (3,)), ("volume_scatter", "u1"), ("pad0", "u1", (3,)), ("pdf_direction_in", "<f4"),
     ("is_delta", "u1"), ("pad1", "u1", (3,)), ("scattering_weight", "<f4", (3,)),
     ("transmittance_weight", "<f4", (3,)), ("direct_contribution", "<f4", (3,)), ("mi_weight", "<f4"),
     ("scattered_contribution", "<f4", (3,)), ("rr_probability", "<f4"), ("eta", "<f4"), ("roughness", "<f4"),
     ("pad2", "<u4"), ("region_ptr", "<u8")])
assert PGL_PATH_SEGMENT_DTYPE.itemsize == 136


def path_segments(num_paths, seed, max_len=12):
    """Random-walk paths of 1..max_len segments in [0, 10]^3 with the mix of
    vertex kinds a path tracer records: delta and glossy vertices (roughness
    spread over [0, 1], a fifth below 0.01), refractive ones (eta != 1),
    volume scattering, zero and partial Russian roulette, lights hit and
    next-event contributions.  Returns (segments, begin) with begin[p] the
    first segment of path p (num_paths + 1 entries)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lens = 1 + np.minimum(np.floor(rng.random(num_paths) * max_len), max_len - 1).astype(np.int64)
    begin = np.zeros(num_paths + 1, dtype=np.uint64)
    begin[1:] = np.cumsum(lens)
    n = int(begin[-1])
    s = np.zeros(n, dtype=PGL_PATH_SEGMENT_DTYPE)
    start = rng.random((num_paths, 3)) * 10.0
    steps = (rng.random((n, 3)) - 0.5) * 3.0
    # walk: cumulative steps within each path (a path's first vertex is its start)
    first = np.zeros(n, dtype=bool)
    first[begin[:-1].astype(np.int64)] = True
    steps[first] = 0.0
    cs = np.cumsum(steps, axis=0)
    pos = np.repeat(start, lens, axis=0) + (cs - np.repeat(cs[first], lens, axis=0))
    s["position"] = pos.astype(np.float32)
    s["direction_in"] = _unit_sphere(rng, n).astype(np.float32)
    s["direction_out"] = _unit_sphere(rng, n).astype(np.float32)
    s["normal"] = _unit_sphere(rng, n).astype(np.float32)
    s["volume_scatter"] = (rng.random(n) < 0.2).astype(np.uint8)
    s["pdf_direction_in"] = (0.01 * det_exp(rng.random(n) * det_log(1000.0))).astype(np.float32)
    s["is_delta"] = (rng.random(n) < 0.1).astype(np.uint8)
    s["scattering_weight"] = (rng.random((n, 3)) * 1.2).astype(np.float32)
    s["transmittance_weight"] = (0.5 + 0.5 * rng.random((n, 3))).astype(np.float32)
    dc = rng.random((n, 3)) * 2.0
    dc[rng.random(n) < 0.5] = 0.0
    s["direct_contribution"] = dc.astype(np.float32)
    s["mi_weight"] = rng.random(n).astype(np.float32)
    sc = rng.random((n, 3))
    sc[rng.random(n) < 0.8] = 0.0
    s["scattered_contribution"] = sc.astype(np.float32)
    rr = rng.random(n)
    u = rng.random(n)
    rr = np.where(u < 0.5, 1.0, np.where(u < 0.6, 0.0, rr))
    s["rr_probability"] = rr.astype(np.float32)
    eta = 1.0 + rng.random(n)
    eta[rng.random(n) < 0.7] = 1.0
    s["eta"] = eta.astype(np.float32)
    rough = rng.random(n)
    rough[rng.random(n) < 0.2] *= 0.01
    s["roughness"] = rough.astype(np.float32)
    return s, begin


def paths_blob(segments, begin, extra=b""):
    """u64 numPaths, u64 begin[numPaths + 1], then the segments."""
    return (np.uint64(len(begin) - 1).tobytes() + np.ascontiguousarray(begin, dtype=np.uint64).tobytes()
            + np.ascontiguousarray(segments).tobytes())
