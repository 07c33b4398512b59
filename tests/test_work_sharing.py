"""CPU models of two warp-level rules of the particle kernels, checked for
every value they hand out (no GPU).

* Work distribution (WarpBatches in jerald_gb300/csrc/common.cuh): warps
  walk units of ub consecutive 32-particle batches; unit u belongs to
  counter region u mod 32; a warp's first unit is static, later ones come
  from its region's counter, the next ticket fetched when a unit starts
  (so a warp that runs out has taken one ticket it never uses). The model
  runs the warps in a random order (the counters' atomics then hand out
  tickets in that order) and checks that every batch of a launch is
  visited exactly once, for launches smaller than one region per warp, with
  partial units and partial batches, and with fewer than 32 warps (the
  grid-stride order).
* Face pairing of the scatters (pair_key / zpair32_flags / pair_keeps in
  jerald_gb300/csrc/common.cuh, used by the paint in csrc/cic.cu and the
  fused adjoint): lane l adds lane l-1's upper-z face to its lower-z corners
  when both stencils do not wrap and lane l's lower corner is lane l-1's plus
  one in z; lane l-1 then skips those four atomics. The model follows each
  corner value symbolically through the shuffles and checks that every value
  of every live lane reaches exactly one atomic, at its own cell. The CIC
  corner setup restates cic_corners (C remainder semantics of
  lib/parops_fast.h:376-409 for out-of-range cells).
"""
import numpy as np
import pytest

REGIONS, UNIT_BATCHES = 32, 16


def _warp_batches(n, nw, rng):
    """Batch bases visited by nw warps over n particles, in a random order."""
    if nw < REGIONS:  # no counters: the grid-stride order
        return [b for w in range(nw) for b in range(32 * w, n, 32 * nw)]
    ub = min(max(n // (32 * 8 * nw), 1), UNIT_BATCHES)
    counter = [0] * REGIONS
    wr = [-(-(nw - r) // REGIONS) for r in range(REGIONS)]  # warps of region r

    def start(r, q):
        return (r + REGIONS * q) * 32 * ub

    def fetch(w):
        r = w % REGIONS
        t = wr[r] + counter[r]
        counter[r] += 1
        return t

    state = {}  # warp -> [base, unit_end, pending]
    visited = []
    todo = list(range(nw))
    while todo:
        i = int(rng.integers(len(todo)))
        w = todo[i]
        if w not in state:  # first(): the static unit, the first ticket
            b = start(w % REGIONS, w // REGIONS)
            state[w] = [b, b + 32 * ub, fetch(w)]
        s = state[w]
        if s[0] >= n:
            todo[i] = todo[-1]
            todo.pop()
            continue
        visited.append(s[0])
        s[0] += 32  # next()
        if s[0] >= s[1]:
            b = start(w % REGIONS, s[2])
            s[0], s[1], s[2] = b, b + 32 * ub, fetch(w)
    return visited


@pytest.mark.parametrize("n,nw", [
    (1, 1), (33, 5), (1000, 31), (1, 32), (31, 32), (32, 33), (5000, 40),
    (288358, 7296),          # 64^3 workload, 912 CTAs of 8 warps: ub = 1
    (2_000_003, 6080),       # ub = 1, a partial last batch
    (3_000_000, 900),        # ub = 13
    (9_000_000, 600),        # ub = 16 (the cap), partial last unit
])
def test_warp_batches_visit_every_batch_once(n, nw):
    rng = np.random.default_rng(n + nw)
    got = np.sort(np.array(_warp_batches(n, nw, rng), dtype=np.int64))
    assert np.array_equal(got, np.arange(0, n, 32, dtype=np.int64))


# reference corner order k -> axis bits (x = bit 0): 000 100 010 001 110 101 011 111
CORNER_BITS = [0, 1, 2, 4, 3, 5, 6, 7]
ZPAIR_HI, ZPAIR_LO = [3, 5, 6, 7], [0, 1, 2, 4]
NO_PAIR = 0xFFFFFFFF


def _corners(i, nm, strides):
    """Per-axis lower/upper offsets of a stencil whose lower cell index is i
    (int(q) per axis), with C remainder semantics outside the mesh."""
    o = []
    for a in range(3):
        n = nm[a]
        if 0 <= i[a] < n:
            lo, hi = i[a], (0 if i[a] + 1 == n else i[a] + 1)
        else:
            c_rem = lambda x: int(np.fmod(x, n))  # noqa: E731  (C %, sign of x)
            lo, hi = abs(c_rem(i[a])), abs(c_rem(c_rem(i[a] + 1)))
        o.append((lo * strides[a], hi * strides[a]))
    return o


def _pair_key(o, strides):
    canon = o[0][1] == o[0][0] + strides[0] and o[1][1] == o[1][0] + strides[1] and o[2][1] == o[2][0] + 1
    return (o[0][0] + o[1][0] + o[2][0]) if canon else NO_PAIR


def _cell(o, bits):
    return o[0][bits & 1] + o[1][(bits >> 1) & 1] + o[2][(bits >> 2) & 1]


def _scatter_model(idx, live, nm):
    """Atomics of one warp: list of (cell, frozenset of (lane, corner))."""
    strides = (nm[1] * nm[2], nm[2], 1)
    cs = [_corners(i, nm, strides) for i in idx]
    key = [(_pair_key(o, strides) if lv else NO_PAIR) for o, lv in zip(cs, live)]
    tz = [l > 0 and key[l] != NO_PAIR and key[l - 1] != NO_PAIR and key[l] == (key[l - 1] + 1) & 0xFFFFFFFF
          for l in range(32)]
    gz = [l < 31 and tz[l + 1] for l in range(32)]
    w = [[{(l, k)} for k in range(8)] for l in range(32)]
    # shuffles read every lane's upper-z values before any lane adds
    up = [[set(w[l][ZPAIR_HI[j]]) for j in range(4)] for l in range(32)]
    for l in range(32):
        if tz[l]:
            for j in range(4):
                w[l][ZPAIR_LO[j]] |= up[l - 1][j]
    atomics = []
    for l in range(32):
        if not live[l]:
            continue
        for k in range(8):
            if k in ZPAIR_LO or not gz[l]:
                atomics.append((_cell(cs[l], CORNER_BITS[k]), frozenset(w[l][k])))
    return atomics, cs, tz


def _check_warp(idx, live, nm):
    atomics, cs, tz = _scatter_model(idx, live, nm)
    seen = {}
    for cell, vals in atomics:
        for (l, k) in vals:
            assert (l, k) not in seen, f"value of lane {l} corner {k} added twice"
            seen[(l, k)] = cell
            assert cell == _cell(cs[l], CORNER_BITS[k]), f"lane {l} corner {k} added at another cell"
    want = {(l, k) for l in range(32) if live[l] for k in range(8)}
    assert set(seen) == want
    return sum(tz)


def test_face_pairing_adds_every_value_once():
    rng = np.random.default_rng(11)
    nm = (8, 6, 10)
    paired = 0
    for trial in range(400):
        kind = trial % 4
        if kind == 0:  # lattice order: z runs along rows, wrapping at the z edge
            s = int(rng.integers(0, 8 * 6 * 10))
            flat = [(s + l) % (8 * 6 * 10) for l in range(32)]
            idx = [(f // 60, (f // 10) % 6, f % 10) for f in flat]
        elif kind == 1:  # random cells, some outside the mesh (negative, = N, beyond)
            idx = [tuple(int(v) for v in rng.integers(-3, (11, 9, 13))) for _ in range(32)]
        elif kind == 2:  # a clump: repeated and neighbouring cells
            c = rng.integers(0, (8, 6, 10))
            idx = [tuple(int(v) for v in (c + rng.integers(0, 2, 3))) for _ in range(32)]
        else:  # runs of z neighbours broken at random
            idx, cur = [], list(rng.integers(0, (8, 6, 10)))
            for _ in range(32):
                if rng.random() < 0.2:
                    cur = list(rng.integers(-1, (9, 7, 11)))
                idx.append(tuple(int(v) for v in cur))
                cur[2] += 1
        nlive = 32 if trial % 5 else int(rng.integers(1, 32))  # a partial last batch
        live = [l < nlive for l in range(32)]
        paired += _check_warp(idx, live, nm)
    assert paired > 1000  # the lattice-order cases do pair
