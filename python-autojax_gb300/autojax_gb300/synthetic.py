"""Seeded synthetic interferometer datasets with the shapes of the benchmark configs.

Host-side input generation (NumPy), not part of the GPU compute path.  The
reference's public dataset (``dataset/data.npz``, built by PyAutoLens) is not
available, so seeded synthetic inputs with the published shapes stand in:

* uv points uniform in the annulus 1e3 <= |uv| <= 5e5 wavelengths;
* per-visibility noise sigma_k ~ lognormal(ln 0.3, 0.5), identical for the
  real and imaginary parts (w_tilde uses the real part only, as in the
  reference's fixtures, tests.py:346-348);
* visibilities: the DFT of a lensed Gaussian source plus N(0, sigma_k^2) noise;
* dirty image consistent with the chi^2 expansion,
  dirty_i = sum_k w_k (Re V_k cos th_ik - Im V_k sin th_ik),
  th_ik = 2 pi (x_i u_k + y_i v_k), x = grid[:, 1], y = grid[:, 0];
* image grid: y decreasing with row, x increasing with column (tests.py:291-302),
  centred on the optical axis;
* source plane: a singular isothermal sphere (SIS) ray-trace, then either a
  rectangular mesh with bilinear weights (4 per row) or Delaunay
  barycentric weights (3 per row) with the mesh's edges as neighbours.

The DFT and the dirty image are computed separably on the regular grid
(two complex GEMMs per K block), so the K = 1e6 configuration builds in
seconds on host cores.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ARCSEC = np.pi / 648000.0


@dataclass(frozen=True)
class Config:
    name: str
    K: int
    grid: int
    pixel_scale: float  # arcsec
    mask_radius: float  # arcsec
    S: int
    mesh: str  # "rect" (bilinear, B=4) or "delaunay" (barycentric, B=3)
    einstein_radius: float = 0.8
    source_radius: float = 1.5
    lam: float = 1.0
    seed: int = 0


CONFIGS = {
    # the small CPU-runnable inversion: K=2e3, 30x30 at 0.1", r=1.2", 16x16 rectangular bilinear source, lam=1
    "cfg1": Config("cfg1", 2_000, 30, 0.1, 1.2, 256, "rect", 0.8, 1.5, 1.0, 101),
    # the mid-size float64 inversion: K=1e5, 80x80 at 0.05", r=2", S=1000 Delaunay
    "cfg2": Config("cfg2", 100_000, 80, 0.05, 2.0, 1_000, "delaunay", 0.8, 1.5, 0.3, 202),
    # the large-K mixed-precision inversion: K=1e6, 100x100 at 0.04", r=2.4", S=1500 Delaunay
    "cfg3": Config("cfg3", 1_000_000, 100, 0.04, 2.4, 1_500, "delaunay", 0.8, 1.5, 1.0, 303),
    # the batched evaluations: K=5e5, ~8000 image pixels (100x100 at 0.04", r=2.0"), S in [500, 2000]
    "cfg5": Config("cfg5", 500_000, 100, 0.04, 2.0, 1_000, "delaunay", 0.8, 1.5, 1.0, 505),
}


def mask_circular(N: int, pixel_scale: float, radius: float) -> np.ndarray:
    """True = masked, following numba.py:50-86 with centre (0, 0)."""
    c = 0.5 * (N - 1)
    ys, xs = np.indices((N, N))
    return (radius * radius) < (np.square((ys - c) * pixel_scale) + np.square((xs - c) * pixel_scale))


def grid_radians_2d(N: int, pixel_scale: float) -> np.ndarray:
    """(N, N, 2) grid in radians, [..., 0] = y (decreasing with row), [..., 1] = x."""
    d = pixel_scale * ARCSEC
    c = 0.5 * (N - 1)
    I, J = np.mgrid[:N, :N]
    g = np.empty((N, N, 2))
    g[:, :, 0] = -d * (I - c)
    g[:, :, 1] = d * (J - c)
    return g


def annulus_uv(rng, K: int, r1: float = 1e3, r2: float = 5e5) -> np.ndarray:
    r = np.sqrt(rng.uniform(r1 * r1, r2 * r2, K))
    th = rng.uniform(0.0, 2.0 * np.pi, K)
    return np.ascontiguousarray(np.stack([r * np.cos(th), r * np.sin(th)], axis=1))


def sis_trace(theta_yx_arcsec: np.ndarray, einstein_radius: float) -> np.ndarray:
    """beta = theta - theta_E theta/|theta| (arcsec), a singular isothermal sphere at the origin."""
    r = np.maximum(np.hypot(theta_yx_arcsec[:, 0], theta_yx_arcsec[:, 1]), 1e-12)
    return theta_yx_arcsec - einstein_radius * theta_yx_arcsec / r[:, None]


def bilinear_mesh(beta: np.ndarray, n: int, half_width: float):
    """Rectangular n x n mesh on [-hw, hw]^2: 4 bilinear weights per traced point, 4-neighbours."""
    h = 2.0 * half_width / (n - 1)
    fy = np.clip((half_width - beta[:, 0]) / h, 0.0, n - 1 - 1e-9)  # row grows downwards (y decreasing)
    fx = np.clip((beta[:, 1] + half_width) / h, 0.0, n - 1 - 1e-9)
    r0 = np.floor(fy).astype(np.int64)
    c0 = np.floor(fx).astype(np.int64)
    ty = fy - r0
    tx = fx - c0
    idx = np.stack([r0 * n + c0, r0 * n + c0 + 1, (r0 + 1) * n + c0, (r0 + 1) * n + c0 + 1], axis=1)
    w = np.stack([(1 - ty) * (1 - tx), (1 - ty) * tx, ty * (1 - tx), ty * tx], axis=1)
    S = n * n
    nb = -np.ones((S, 4), dtype=np.int64)
    for s in range(S):
        r, c = divmod(s, n)
        lst = [q for q, ok in ((s - n, r > 0), (s - 1, c > 0), (s + 1, c < n - 1), (s + n, r < n - 1)) if ok]
        nb[s, : len(lst)] = lst
    return np.ascontiguousarray(idx), np.ascontiguousarray(w), nb


def delaunay_mesh(beta: np.ndarray, points: np.ndarray):
    """Barycentric weights of each traced point in the Delaunay triangulation of ``points``.

    Points outside the hull map to their nearest mesh vertex with weight 1 and
    the row is -1 padded (a ragged row, as the reference's format allows).
    """
    from scipy.spatial import Delaunay, cKDTree

    tri = Delaunay(points)
    simplex = tri.find_simplex(beta)
    M = beta.shape[0]
    idx = -np.ones((M, 3), dtype=np.int64)
    w = np.zeros((M, 3))
    inside = simplex >= 0
    Tm = tri.transform[simplex[inside]]
    bary2 = np.einsum("nij,nj->ni", Tm[:, :2, :], beta[inside] - Tm[:, 2, :])
    bary = np.concatenate([bary2, 1.0 - bary2.sum(axis=1, keepdims=True)], axis=1)
    idx[inside] = tri.simplices[simplex[inside]]
    w[inside] = bary
    if (~inside).any():
        _, near = cKDTree(points).query(beta[~inside])
        idx[~inside, 0] = near
        w[~inside, 0] = 1.0
    indptr, indices = tri.vertex_neighbor_vertices
    deg = np.diff(indptr)
    P = int(deg.max())
    nb = -np.ones((points.shape[0], P), dtype=np.int64)
    for s in range(points.shape[0]):
        nb[s, : deg[s]] = np.sort(indices[indptr[s] : indptr[s + 1]])
    return np.ascontiguousarray(idx), np.ascontiguousarray(w), nb


def _dft_and_dirty(image_2d, g2d, uv, w, rng, sigma, block=16384):
    """Separable DFT of a gridded image and the consistent dirty image.

    V_k = sum_ij I_ij exp(-2 pi i (x_j u_k + y_i v_k)); with x_j = x0 + d j and
    y_i = y0 - d i the sum factorises into two complex GEMMs per block.
    """
    N = image_2d.shape[0]
    d = g2d[0, 1, 1] - g2d[0, 0, 1]
    x0 = g2d[0, 0, 1]
    y0 = g2d[0, 0, 0]
    K = uv.shape[0]
    vis = np.empty(K, dtype=np.complex128)
    dirty = np.zeros((N, N))
    j = np.arange(N)
    for k0 in range(0, K, block):
        k1 = min(K, k0 + block)
        u = uv[k0:k1, 0]
        v = uv[k0:k1, 1]
        Eu = np.exp(-2j * np.pi * d * np.outer(u, j))  # (k, col)
        Ev = np.exp(2j * np.pi * d * np.outer(v, j))  # (k, row): y_i = y0 - d i
        ph0 = np.exp(-2j * np.pi * (x0 * u + y0 * v))
        inner = image_2d @ Eu.T  # (row, k)
        V = ph0 * np.einsum("kr,rk->k", Ev, inner)
        V = V + sigma[k0:k1] * (rng.standard_normal(k1 - k0) + 1j * rng.standard_normal(k1 - k0))
        vis[k0:k1] = V
        c = w[k0:k1] * V * np.conj(ph0)
        # dirty_rc = Re sum_k c_k exp(+2 pi i (x_c u_k + y_r v_k)) without the x0/y0 phase (folded into c)
        dirty += np.real((np.conj(Ev).T * c) @ np.conj(Eu))
    return vis, dirty


def make_dataset(cfg: Config | str, *, K: int | None = None, S: int | None = None, seed: int | None = None) -> dict:
    """Build every array the inversion needs for one configuration.

    ``K``/``S``/``seed`` override the configuration's values (smaller parity cases).
    Returns a dict keyed by the reference's parameter names.
    """
    if isinstance(cfg, str):
        cfg = CONFIGS[cfg]
    K = cfg.K if K is None else int(K)
    S = cfg.S if S is None else int(S)
    rng = np.random.default_rng(cfg.seed if seed is None else seed)
    N = cfg.grid
    mask = mask_circular(N, cfg.pixel_scale, cfg.mask_radius)
    native = np.ascontiguousarray(np.argwhere(~mask).astype(np.int64))
    g2d = grid_radians_2d(N, cfg.pixel_scale)
    slim = np.ascontiguousarray(g2d[~mask])
    M = slim.shape[0]

    uv = annulus_uv(rng, K)
    sigma = np.exp(np.log(0.3) + 0.5 * rng.standard_normal(K))
    w = 1.0 / sigma**2
    noise_map = np.ascontiguousarray(sigma + 1j * sigma)

    theta = slim / ARCSEC  # (M, 2) arcsec, (y, x)
    beta = sis_trace(theta, cfg.einstein_radius)
    if cfg.mesh == "rect":
        n = int(round(np.sqrt(S)))
        half = float(np.abs(beta).max()) * 1.0001
        pidx, pw, nb = bilinear_mesh(beta, n, half)
        S = n * n
    else:
        rr = cfg.source_radius * np.sqrt(rng.uniform(0, 1, S))
        tt = rng.uniform(0, 2 * np.pi, S)
        pts = np.stack([rr * np.sin(tt), rr * np.cos(tt)], axis=1)
        pidx, pw, nb = delaunay_mesh(beta, pts)
    nsz = (nb != -1).sum(axis=1).astype(np.int64)

    # lensed Gaussian source (0.25" sigma, offset 0.1") seen in the image plane
    src = np.exp(-0.5 * (np.square(beta[:, 0] - 0.1) + np.square(beta[:, 1] - 0.05)) / 0.25**2)
    img = np.zeros((N, N))
    img[~mask] = src * 0.05
    vis, dirty2d = _dft_and_dirty(img, g2d, uv, w, rng, sigma)
    return {
        "config": cfg.name,
        "grid_size": N,
        "pixel_scale": cfg.pixel_scale,
        "real_space_mask": mask,
        "native_index_for_slim_index": native,
        "grid_radians_2d": g2d,
        "grid_radians_slim": slim,
        "uv_wavelengths": uv,
        "noise_map": noise_map,
        "noise_map_real": np.ascontiguousarray(noise_map.real),
        "data": np.ascontiguousarray(vis),
        "visibilities_real": np.ascontiguousarray(vis.real),
        "dirty_image": np.ascontiguousarray(dirty2d[~mask]),
        "pix_indexes_for_sub_slim_index": pidx,
        "pix_weights_for_sub_slim_index": pw,
        "neighbors": nb,
        "neighbors_sizes": nsz,
        "pixels": int(S),
        "coefficient": float(np.sqrt(cfg.lam)),
        "M": M,
        "K": K,
        "S": int(S),
    }


def lens_models(d: dict, n: int, *, S_range=(500, 2000), einstein_range=(0.6, 1.2), lam_range=(1e-3, 1e3),
                seed: int = 0) -> list[dict]:
    """``n`` lens models for one dataset, as a sampler would propose them.

    Each model draws its source-pixel count S uniformly from ``S_range``, its
    SIS Einstein radius uniformly from ``einstein_range`` and lambda
    log-uniformly from ``lam_range``.  Its S Delaunay vertices are traced
    image pixels (a random subset, jittered by 1e-4"), as image-plane-derived
    meshes place them, so every source pixel has data nearby; the image grid
    is ray-traced and mapped with barycentric weights of their triangulation.
    """
    rng = np.random.default_rng(seed)
    theta = d["grid_radians_slim"] / ARCSEC
    out = []
    for _ in range(n):
        S = int(rng.integers(S_range[0], S_range[1] + 1))
        theta_e = float(rng.uniform(*einstein_range))
        lam = float(np.exp(rng.uniform(np.log(lam_range[0]), np.log(lam_range[1]))))
        beta = sis_trace(theta, theta_e)
        pick = rng.choice(beta.shape[0], size=min(S, beta.shape[0]), replace=False)
        pts = beta[pick] + 1e-4 * rng.standard_normal((pick.size, 2))
        S = pick.size
        pidx, pw, nb = delaunay_mesh(beta, pts)
        out.append({
            "S": S,
            "einstein_radius": theta_e,
            "coefficient": float(np.sqrt(lam)),
            "pix_indexes_for_sub_slim_index": pidx,
            "pix_weights_for_sub_slim_index": pw,
            "neighbors": nb,
            "neighbors_sizes": (nb != -1).sum(axis=1).astype(np.int64),
        })
    return out

