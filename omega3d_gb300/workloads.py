"""Seeded synthetic scenes with the shapes, sizes and value distributions of the
Biot-Savart / BEM workloads this library is measured on.  All arrays are float32,
component-major SoA ([3, n] positions/strengths, [n] radii), numpy on the host.

None of these reproduces a published data set: they are generated from fixed seeds.
"""
import numpy as np


def vortex_ring(n=16384, seed=1, major=1.0, minor=0.1, sigma=0.05):
    """Thin vortex ring: n particles uniform in the volume of a torus (major radius
    `major`, cross-section radius `minor`), strength vectors tangent to the ring's
    azimuth with magnitude 1/n, all core radii `sigma`."""
    rng = np.random.default_rng(seed)
    pts = []
    need = n
    while need > 0:
        m = max(4 * need, 1024)
        x = rng.uniform(-(major + minor), major + minor, m)
        y = rng.uniform(-(major + minor), major + minor, m)
        z = rng.uniform(-minor, minor, m)
        rr = np.sqrt(x * x + y * y)
        keep = (rr - major) ** 2 + z * z < minor * minor
        pts.append(np.stack([x[keep], y[keep], z[keep]]))
        need -= int(keep.sum())
    p = np.concatenate(pts, axis=1)[:, :n]
    rr = np.sqrt(p[0] ** 2 + p[1] ** 2)
    s = np.stack([-p[1] / rr, p[0] / rr, np.zeros(n)]) / n
    r = np.full(n, sigma)
    return p.astype(np.float32), s.astype(np.float32), r.astype(np.float32)


def gaussian_cloud(n=262144, seed=2, pos_std=0.3, str_scale=1e-3, rmin=0.01, rmax=0.03):
    """Particle cloud: positions N(0, pos_std^2) per axis, strength components
    i.i.d. N(0,1)*str_scale, core radii uniform in [rmin, rmax]."""
    rng = np.random.default_rng(seed)
    x = rng.normal(0.0, pos_std, (3, n))
    s = rng.normal(0.0, 1.0, (3, n)) * str_scale
    r = rng.uniform(rmin, rmax, n)
    return x.astype(np.float32), s.astype(np.float32), r.astype(np.float32)


def shell_particles(n=100000, seed=3, rin=1.02, rout=1.5, str_scale=1e-3, sigma=0.02):
    """Particles uniform in the spherical shell rin < r < rout."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, n)
    rad = (rin ** 3 + u * (rout ** 3 - rin ** 3)) ** (1.0 / 3.0)
    d = rng.normal(0.0, 1.0, (3, n))
    d /= np.linalg.norm(d, axis=0)
    x = d * rad
    s = rng.normal(0.0, 1.0, (3, n)) * str_scale
    r = np.full(n, sigma)
    return x.astype(np.float32), s.astype(np.float32), r.astype(np.float32)


def wake_particles(n=1048576, seed=5, xmin=1.0, xmax=6.0, half=1.5, str_scale=1e-3, sigma=0.015):
    """Particles uniform in the box x in [xmin, xmax], |y|, |z| < half."""
    rng = np.random.default_rng(seed)
    x = np.stack([rng.uniform(xmin, xmax, n), rng.uniform(-half, half, n), rng.uniform(-half, half, n)])
    s = rng.normal(0.0, 1.0, (3, n)) * str_scale
    r = np.full(n, sigma)
    return x.astype(np.float32), s.astype(np.float32), r.astype(np.float32)


def batch_systems(nsys=64, seed=4, nmin=1024, nmax=65536, nfield=4096):
    """Independent systems with log-uniform sizes; each a Gaussian blob (blob sigma
    uniform in [0.1, 0.5]) with N(0, 1e-3^2) strength components, core radii uniform
    in [0.01, 0.05], plus nfield field points on a jittered 16^3 grid spanning +-2 sigma."""
    rng = np.random.default_rng(seed)
    systems = []
    side = int(round(nfield ** (1.0 / 3.0)))
    for _ in range(nsys):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        sb = rng.uniform(0.1, 0.5)
        x = rng.normal(0.0, sb, (3, n))
        s = rng.normal(0.0, 1.0, (3, n)) * 1e-3
        r = rng.uniform(0.01, 0.05, n)
        g = np.linspace(-2 * sb, 2 * sb, side)
        sp = g[1] - g[0]
        gx, gy, gz = np.meshgrid(g, g, g, indexing="ij")
        f = np.stack([gx.ravel(), gy.ravel(), gz.ravel()])[:, :nfield]
        f = f + rng.uniform(-0.25, 0.25, f.shape) * sp
        systems.append((x.astype(np.float32), s.astype(np.float32), r.astype(np.float32), f.astype(np.float32)))
    return systems


def lattice_particles(k=64, seed=6, spacing=0.01, jitter=0.35, str_scale=1e-4, overlap=1.5, elong_scale=0.12):
    """k^3 particles on a cubic lattice of the nominal separation `spacing`, each moved by
    N(0, (jitter*spacing)^2) per axis, core radius overlap*spacing, strengths
    (2, 0, 0)*str_scale plus N(0,1)*str_scale per component, elongations 1 + Exp(elong_scale):
    the state the split and merge operators see after some stretching steps (with the
    default tail about 19 % of the particles exceed the split threshold 1.2, and about 9 %
    have a neighbour closer than half a separation)."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), 0).reshape(3, -1).astype(np.float64) * spacing
    g += rng.normal(scale=jitter * spacing, size=g.shape)
    s = rng.normal(size=g.shape) * str_scale
    s[0] += 2.0 * str_scale
    r = np.full(g.shape[1], overlap * spacing)
    e = 1.0 + rng.exponential(elong_scale, g.shape[1])
    return g.astype(np.float32), s.astype(np.float32), r.astype(np.float32), e.astype(np.float32)


def duplicated_particles(k=12, seed=41, every=5, seed_dup=2):
    """lattice_particles(k, seed) followed by exact copies of a seeded 1/every of its
    particles (same position, radius and elongation; new strengths N(0,1)*1e-4): neighbours
    at exactly equal distance, the case where the order of a radius search's ties decides
    which of two coincident particles a merge keeps."""
    x, s, r, e = lattice_particles(k=k, seed=seed)
    rng = np.random.default_rng(seed_dup)
    n = x.shape[1]
    d = np.sort(rng.choice(n, n // every, replace=False))
    sd = (rng.normal(size=(3, d.size)) * 1e-4).astype(np.float32)
    cat = lambda a, b: np.ascontiguousarray(np.concatenate([a, b], axis=-1))
    return cat(x, x[:, d]), cat(s, sd), cat(r, r[d]), cat(e, e[d])
