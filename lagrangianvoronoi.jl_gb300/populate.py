"""Host-side seed generators: the `populate_*!` family of the reference
(src/populate.jl:18-179) restated in numpy, plus the seeded jittered lattice
used by the benchmark workloads.

The reference generates seeds on the host, pushes them into the grid and then
calls `remesh!` before applying the user's `ic!`; the GPU grid does the same:
positions are produced here, uploaded once, and meshed on the device.
"""
import numpy as np

_MASK = (1 << 64) - 1


def splitmix64(seed, count):
    """SplitMix64 stream (Steele, Lea & Flood 2014): `count` uint64 values.

    Integer-only, so the jitter is bit-identical on every host."""
    out = np.empty(count, dtype=np.uint64)
    s = seed & _MASK
    # vectorised: state_k = seed + (k+1)*golden (mod 2^64)
    k = np.arange(1, count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(s) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    out[:] = z
    return out


def uniform01(seed, count):
    """Doubles in [0, 1) from the top 53 bits of SplitMix64."""
    return (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def jittered_lattice(xlims, ylims, nx, ny, jitter=0.1, seed=12345):
    """nx*ny seeds x_ij = ((i - 1/2) hx + xi1, (j - 1/2) hy + xi2) with
    xi ~ U(-jitter*h, jitter*h); seed order is row-major in y then x
    (index = j*nx + i)."""
    hx = (xlims[1] - xlims[0]) / nx
    hy = (ylims[1] - ylims[0]) / ny
    u = uniform01(seed, 2 * nx * ny).reshape(ny * nx, 2)
    ii = np.tile(np.arange(nx, dtype=np.float64), ny)
    jj = np.repeat(np.arange(ny, dtype=np.float64), nx)
    x = xlims[0] + (ii + 0.5) * hx + (2.0 * u[:, 0] - 1.0) * (jitter * hx)
    y = ylims[0] + (jj + 0.5) * hy + (2.0 * u[:, 1] - 1.0) * (jitter * hy)
    return np.ascontiguousarray(np.stack([x, y], axis=1))


def _inside(xlims, ylims, p):
    return (xlims[0] <= p[:, 0]) & (p[:, 0] <= xlims[1]) & (ylims[0] <= p[:, 1]) & (p[:, 1] <= ylims[1])


def rect_seeds(xlims, ylims, dr, charfun=None):
    """populate_rect! (src/populate.jl:50-57): range(xmin, xmax, N) + dr/2,
    which leaves the last row and column outside the domain."""
    N = int(round((xlims[1] - xlims[0]) / dr))
    M = int(round((ylims[1] - ylims[0]) / dr))
    pts = []
    for x1 in np.linspace(xlims[0], xlims[1], N):
        for x2 in np.linspace(ylims[0], ylims[1], M):
            pts.append((x1 + 0.5 * dr, x2 + 0.5 * dr))
    return _filter(xlims, ylims, np.array(pts, dtype=np.float64).reshape(-1, 2), charfun)


def hex_seeds(xlims, ylims, dr, charfun=None):
    """populate_hex! (src/populate.jl:155-179)."""
    a = (4.0 / 3.0) ** 0.25 * dr
    b = (3.0 / 4.0) ** 0.25 * dr
    i_min = int(np.floor(xlims[0] / a)) - 1
    j_min = int(np.floor(ylims[0] / b))
    i_max = int(np.ceil(xlims[1] / a))
    j_max = int(np.ceil(ylims[1] / b))
    pts = []
    for i in range(i_min, i_max + 1):
        for j in range(j_min, j_max + 1):
            # Julia's j % 2 keeps the sign of j (rem), as does math.fmod
            jm = j % 2 if j >= 0 else -((-j) % 2)
            pts.append(((i + jm / 2) * a, j * b))
    return _filter(xlims, ylims, np.array(pts, dtype=np.float64).reshape(-1, 2), charfun)


def circ_seeds(xlims, ylims, dr, center=(0.0, 0.0), charfun=None):
    """populate_circ! (src/populate.jl:18-35)."""
    c = np.asarray(center, dtype=np.float64)
    corners = np.array([[xlims[0], ylims[0]], [xlims[0], ylims[1]], [xlims[1], ylims[1]], [xlims[1], ylims[0]]])
    r_max = np.max(np.linalg.norm(corners - c, axis=1))
    pts = []
    r = 0.5 * dr
    while r <= r_max:
        k_max = int(round(2.0 * np.pi * r / dr))
        for k in range(1, k_max + 1):
            th = 2.0 * np.pi * k / k_max
            pts.append((c[0] + r * np.cos(th), c[1] + r * np.sin(th)))
        r += dr
    return _filter(xlims, ylims, np.array(pts, dtype=np.float64).reshape(-1, 2), charfun)


def rand_seeds(xlims, ylims, dr, seed=1, charfun=None):
    """populate_rand! (src/populate.jl:75-91) with a seeded generator."""
    N = int(round(abs(xlims[1] - xlims[0]) * abs(ylims[1] - ylims[0]) / dr ** 2))
    u = uniform01(seed, 2 * N).reshape(N, 2)
    x = u[:, 0] * xlims[1] + (1 - u[:, 0]) * xlims[0]
    y = u[:, 1] * ylims[1] + (1 - u[:, 1]) * ylims[0]
    return _filter(xlims, ylims, np.stack([x, y], axis=1), charfun)


def vogel_seeds(xlims, ylims, dr, center=(0.0, 0.0), charfun=None):
    """populate_vogel! (src/populate.jl:103-119)."""
    c = np.asarray(center, dtype=np.float64)
    corners = np.array([[xlims[0], ylims[0]], [xlims[0], ylims[1]], [xlims[1], ylims[1]], [xlims[1], ylims[0]]])
    r_max = np.max(np.linalg.norm(corners - c, axis=1))
    N = int(round(np.pi * r_max * r_max / dr ** 2))
    i = np.arange(1, N + 1, dtype=np.float64)
    r = r_max * np.sqrt(i / N)
    th = 2.39996322972865332 * i
    pts = np.stack([c[0] + r * np.cos(th), c[1] + r * np.sin(th)], axis=1)
    return _filter(xlims, ylims, pts, charfun)


def _filter(xlims, ylims, pts, charfun):
    keep = _inside(xlims, ylims, pts)
    if charfun is not None:
        keep &= np.array([bool(charfun(p)) for p in pts], dtype=bool)
    return np.ascontiguousarray(pts[keep])
