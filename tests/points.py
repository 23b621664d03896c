"""Coordinate sets for the index-map tests: random, adversarial (a few ulps
around every cell edge, the poles and the phi = 0 / 2pi seam), and the
staggered grid points themselves."""
import numpy as np


def _ulp_cloud(centres, k=3):
    c = np.asarray(centres, np.float32)
    out = [c]
    up, dn = c.copy(), c.copy()
    for _ in range(k):
        up = np.nextafter(up, np.float32(np.inf))
        dn = np.nextafter(dn, np.float32(-np.inf))
        out += [up.copy(), dn.copy()]
    return np.concatenate(out)


def index_points(nt, n_random=200000, seed=0):
    rng = np.random.default_rng(seed)
    h = np.float32(np.pi / nt)
    hd = np.float64(h)
    # random over a range that exercises both wraps
    phi_r = rng.uniform(-2 * np.pi, 4 * np.pi, n_random).astype(np.float32)
    th_r = rng.uniform(-np.pi, 2 * np.pi, n_random).astype(np.float32)
    # cell edges of all three staggerings, +-3 ulps, in both coordinates
    edges = np.concatenate([np.arange(-2, 2 * nt + 3) * hd + off * hd for off in (0.0, 0.5, -0.5, 1.0)])
    ecloud = _ulp_cloud(edges)
    specials = _ulp_cloud([0.0, np.pi, 2 * np.pi, -np.pi, 3 * np.pi, np.pi / 2, -0.0, 4 * np.pi], k=8)
    ph_e = rng.choice(ecloud, 100000)
    th_e = rng.uniform(0, np.pi, 100000).astype(np.float32)
    th_e2 = rng.choice(ecloud, 100000)
    ph_e2 = rng.uniform(0, 2 * np.pi, 100000).astype(np.float32)
    sp = np.array(np.meshgrid(specials, specials)).reshape(2, -1).astype(np.float32)
    # the grid points the kernels themselves sample at
    i = np.arange(2 * nt, dtype=np.float32)
    j = np.arange(nt, dtype=np.float32)
    gp = []
    for po, to in ((-0.5, 0.5), (0.0, 1.0), (0.0, 0.5)):
        P, T = np.meshgrid((i + np.float32(po)) * h, (j + np.float32(to)) * h)
        gp.append(np.stack([P.ravel(), T.ravel()]))
    gp = np.concatenate(gp, axis=1).astype(np.float32)
    phi = np.concatenate([phi_r, ph_e, ph_e2, sp[0], gp[0]]).astype(np.float32)
    theta = np.concatenate([th_r, th_e, th_e2, sp[1], gp[1]]).astype(np.float32)
    return phi, theta
