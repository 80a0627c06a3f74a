"""Initial conditions and drivers shared by the parity tests and bench.py.

Cell centres follow samurai's Cell::center(): origin + length * (index + 0.5)
(cell.hpp:130-138) with the unit box origin 0 and length 2^-level.
"""
import numpy as np


def centers(level, coords):
    length = 1.0 / np.left_shift(1, level.astype(np.int64)).astype(np.float64)
    return length[:, None] * (coords.astype(np.float64) + 0.5)


def disc(level, coords, xc=0.3, yc=0.3, radius=0.2):
    """demos/FiniteVolume/advection_2d.cpp:22-44"""
    c = centers(level, coords)
    inside = ((c[:, 0] - xc) * (c[:, 0] - xc) + (c[:, 1] - yc) * (c[:, 1] - yc)) <= radius * radius
    return np.where(inside, 1.0, 0.0)


def readme_square(level, coords, length=0.2):
    """README.md:110-118: u = 1 where |center - 0.5| <= length/2 in every direction"""
    c = centers(level, coords)
    inside = np.all(np.abs(c - 0.5) <= 0.5 * length, axis=1)
    return np.where(inside, 1.0, 0.0)


class SplitMix64:
    """Fixed-algorithm RNG (SplitMix64) with a 53-bit uniform mapping, so the
    synthetic inputs do not depend on a library's distribution code."""

    def __init__(self, seed):
        self.s = np.uint64(seed)

    def next_u64(self):
        with np.errstate(over="ignore"):
            self.s = np.uint64(self.s + np.uint64(0x9E3779B97F4A7C15))
            z = self.s
            z = np.uint64((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9))
            z = np.uint64((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB))
            return np.uint64(z ^ (z >> np.uint64(31)))

    def uniform(self, lo=0.0, hi=1.0):
        u = float(self.next_u64() >> np.uint64(11)) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u


def shapes_2d(seed, n_squares=16, n_gauss=16):
    """Seeded sum of indicator squares and Gaussians (the max_level-12 2D
    workload: side U[0.02,0.1], centre U[0.2,0.8]^2, amplitude U[0.5,1],
    Gaussian sigma U[0.005,0.03], centre U[0.2,0.8]^2, amplitude U[0.5,1])."""
    rng = SplitMix64(seed)
    sq = []
    for _ in range(n_squares):
        side = rng.uniform(0.02, 0.1)
        cx, cy = rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8)
        amp = rng.uniform(0.5, 1.0)
        sq.append((side, cx, cy, amp))
    ga = []
    for _ in range(n_gauss):
        sig = rng.uniform(0.005, 0.03)
        cx, cy = rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8)
        amp = rng.uniform(0.5, 1.0)
        ga.append((sig, cx, cy, amp))

    def f(level, coords):
        c = centers(level, coords)
        u = np.zeros(len(c))
        for side, cx, cy, amp in sq:
            inside = (np.abs(c[:, 0] - cx) <= 0.5 * side) & (np.abs(c[:, 1] - cy) <= 0.5 * side)
            u = u + np.where(inside, amp, 0.0)
        for sig, cx, cy, amp in ga:
            r2 = (c[:, 0] - cx) * (c[:, 0] - cx) + (c[:, 1] - cy) * (c[:, 1] - cy)
            u = u + amp * np.exp(-r2 / (2.0 * sig * sig))
        return u

    return f


def shape_sum_2d(squares, gaussians):
    """u0 = sum of indicator squares (side, cx, cy, amp) and Gaussians (sigma, cx, cy, amp)."""

    def f(level, coords):
        c = centers(level, coords)
        u = np.zeros(len(c))
        for side, cx, cy, amp in squares:
            inside = (np.abs(c[:, 0] - cx) <= 0.5 * side) & (np.abs(c[:, 1] - cy) <= 0.5 * side)
            u = u + np.where(inside, amp, 0.0)
        for sig, cx, cy, amp in gaussians:
            r2 = (c[:, 0] - cx) * (c[:, 0] - cx) + (c[:, 1] - cy) * (c[:, 1] - cy)
            u = u + amp * np.exp(-r2 / (2.0 * sig * sig))
        return u

    return f


def batch_instances(seed, n, max_levels=(7, 11), min_level=2):
    """Seeded independent 2D problems for the batched mode: max_level
    U{7..11}, min_level 2, a U[-1,1]^2, 1-8 shapes (squares or Gaussians with
    the distributions of shapes_2d), eps in {1e-3, 1e-4}, regularity 2,
    dt = 0.5 * 2^-max_level (stable for |a_x| + |a_y| <= 2)."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(n):
        lo, hi = max_levels
        maxl = lo + min(hi - lo, int(rng.uniform() * (hi - lo + 1)))
        a = (rng.uniform(-1.0, 1.0), rng.uniform(-1.0, 1.0))
        n_shapes = 1 + min(7, int(rng.uniform() * 8))
        squares, gaussians = [], []
        for _ in range(n_shapes):
            if rng.uniform() < 0.5:
                squares.append((rng.uniform(0.02, 0.1), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.5, 1.0)))
            else:
                gaussians.append((rng.uniform(0.005, 0.03), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.5, 1.0)))
        eps = 1e-3 if rng.uniform() < 0.5 else 1e-4
        out.append(
            dict(
                min_level=min_level,
                max_level=maxl,
                a=a,
                eps=eps,
                regularity=2.0,
                dt=0.5 / (1 << maxl),
                u0=shape_sum_2d(squares, gaussians),
            )
        )
    return out


def ball_3d(seed, n_gauss=8):
    """Seeded ball indicator (radius U[0.1,0.2], centre U[0.3,0.7]^3) plus
    Gaussians (sigma U[0.01,0.05], centre U[0.3,0.7]^3, amplitude U[0.5,1])."""
    rng = SplitMix64(seed)
    rad = rng.uniform(0.1, 0.2)
    bc = [rng.uniform(0.3, 0.7) for _ in range(3)]
    ga = []
    for _ in range(n_gauss):
        sig = rng.uniform(0.01, 0.05)
        cc = [rng.uniform(0.3, 0.7) for _ in range(3)]
        amp = rng.uniform(0.5, 1.0)
        ga.append((sig, cc, amp))

    def f(level, coords):
        c = centers(level, coords)
        r2 = sum((c[:, d] - bc[d]) * (c[:, d] - bc[d]) for d in range(3))
        u = np.where(r2 <= rad * rad, 1.0, 0.0)
        for sig, cc, amp in ga:
            r2 = sum((c[:, d] - cc[d]) * (c[:, d] - cc[d]) for d in range(3))
            u = u + amp * np.exp(-r2 / (2.0 * sig * sig))
        return u

    return f


def demo_time_loop(sim, dt, Tf, eps, regularity, a, scheme=0):
    """The time loop of demos/FiniteVolume/advection_2d.cpp:124-156 (adapt,
    clipped time step, ghost update, upwind), on any object exposing
    adapt/update_ghost/upwind.  Returns the number of steps."""
    t = 0.0
    nt = 0
    while t != Tf:
        sim.adapt(eps, regularity)
        t += dt
        if t > Tf:
            dt += Tf - t
            t = Tf
        sim.update_ghost()
        sim.upwind(a, dt, scheme)
        nt += 1
    return nt


def gaussian_target(seed):
    """Seeded Gaussian target of the adjoint workload: centre U[0.3,0.7]^2,
    sigma U[0.05,0.15], amplitude 1."""
    rng = SplitMix64(seed)
    cx, cy = rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7)
    sig = rng.uniform(0.05, 0.15)

    def f(level, coords):
        c = centers(level, coords)
        r2 = (c[:, 0] - cx) * (c[:, 0] - cx) + (c[:, 1] - cy) * (c[:, 1] - cy)
        return np.exp(-r2 / (2.0 * sig * sig))

    return f


def cell_volumes(level, dim=2):
    return np.ldexp(1.0, -dim * level.astype(np.int64))


def save_mesh_arrays(level, coords, max_level):
    """Points and connectivity of samurai::save for leaf cells in for_each_cell
    order (io/hdf5.hpp:85-144, extract_coords_and_connectivity): the corners of
    each cell in the element order of get_element (hdf5.hpp:64-83) receive ids
    in order of first appearance; points are (x, y, z) with z = 0 in 2D."""
    level = np.asarray(level).astype(np.int64)
    coords = np.asarray(coords).astype(np.int64)
    dim = coords.shape[1]
    if dim == 2:
        elem = [(0, 0), (1, 0), (1, 1), (0, 1)]
    else:
        elem = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    shift = (max_level - level)[:, None]
    keys = np.stack([(coords + np.array(e, np.int64)) << shift for e in elem], axis=1).reshape(-1, dim)
    span = (1 << max_level) + 1
    scalar = keys[:, 0] + span * keys[:, 1] + (span * span * keys[:, 2] if dim == 3 else 0)
    _, first, inverse = np.unique(scalar, return_index=True, return_inverse=True)
    order = np.argsort(first)
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    connectivity = rank[inverse.reshape(-1)].reshape(len(level), len(elem)).astype(np.uint64)
    points = np.zeros((len(order), 3))
    points[:, :dim] = np.ldexp(keys[first[order]].astype(np.float64), -max_level)
    return points, connectivity


def level_cell_array(rows, dim):
    """LevelCellArray layout of one level (level_cell_array.hpp:1005-1077,
    init_from_level_cell_list) from its x-intervals given row by row in
    for_each_interval order as records (start, end, y[, z], index).  Returns
    (intervals, offsets): intervals[d] lists (start, end, index) along
    dimension d, offsets[d - 1] the offsets of dimension d >= 1.  A direct
    restatement of the recursion: along dimension N >= 1 each coordinate of a
    non-empty sub-grid continues the working interval when it is adjacent, or
    starts one with index = len(offsets) - coordinate; offsets record the
    size of the dimension below before the sub-grid is added, and a final
    entry closes each offsets list."""
    intervals = [[] for _ in range(dim)]
    offsets = [[] for _ in range(dim - 1)]
    # nested grid: coordinate -> sub-grid, the innermost holding x-intervals
    grid = {}
    for r in rows:
        key = (int(r[3]), int(r[2])) if dim == 3 else (int(r[2]),)
        node = grid
        for k in key[:-1]:
            node = node.setdefault(k, {})
        node.setdefault(key[-1], []).append((int(r[0]), int(r[1]), int(r[dim + 1])))

    def build(node, n):
        cur = None
        for coord in sorted(node):
            prev = len(intervals[n - 1])
            if n - 1 == 0:
                intervals[0].extend(node[coord])
            else:
                build(node[coord], n - 1)
            if cur is not None and coord == cur[1]:
                cur[1] += 1
            else:
                if cur is not None:
                    intervals[n].append(tuple(cur))
                cur = [coord, coord + 1, len(offsets[n - 1]) - coord]
            offsets[n - 1].append(prev)
        if cur is not None:
            intervals[n].append(tuple(cur))

    if rows is not None and len(rows):
        build(grid, dim - 1)
        for d in range(dim - 1):
            offsets[d].append(len(intervals[d]))
    return intervals, offsets
