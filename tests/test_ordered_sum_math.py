"""The method of the GPU's reference-order sums (csrc/ordered.cu), checked on
the CPU in Python integers: per-binade element functions of the running sum's
parity, their in-order composition, one thread's fold of a chunk, binade
predictions from approximate prefix sums, aggregate levels, the walker that
skips empty runs, applies runs and replays chunks, and the integer replay,
against plain sequential f64 addition (metrics.rs:215-224 adds one value after
the other).  Chunk size and fan-out are small here so that every level and
every replay path is exercised."""

import math
import random

import numpy as np
import pytest

TWO53 = 1 << 53
SAT = 1 << 54
INVALID = None


def sat(a):
    return SAT if a >= SAT else a


def binade(s):
    return math.frexp(s)[1] - 1  # s in [2^E, 2^(E+1))


def units(s):
    E = binade(s)
    return int(math.ldexp(s, 52 - E)), E


def from_units(u, E):
    return math.ldexp(float(u), E - 52)


# a function: (i0, i1, o0, o1, E) with E = "any" for the identity valid everywhere
IDENT = (0, 0, 0, 1, "any")


def elem_fn(M, k, E):
    if M == 0:
        return IDENT
    shift = (E - 52) - k
    if shift <= 0:
        a = sat(M << -shift)
        return (a, a, a & 1, (a & 1) ^ 1, E)
    if shift >= 64:
        return (0, 0, 0, 1, E)
    a, rem, half = M >> shift, M & ((1 << shift) - 1), 1 << (shift - 1)
    if rem != half:
        a += rem > half
        return (a, a, a & 1, (a & 1) ^ 1, E)
    odd = a & 1
    return (a + odd, a + (odd ^ 1), 0, 0, E)


def acc_chunk(terms, E, mbits):
    """A chunk's function folded value by value, as one GPU thread does it
    (ordered.cu acc_elem): increments and parities for input parity 0 and 1."""
    i0 = i1 = 0
    o0, o1 = 0, 1
    em52 = E - 52
    for M, k in terms:
        if M == 0:
            continue
        sh = em52 - k
        if sh <= 0:
            c = SAT if (sh <= -54 or (M >> (54 + sh)) != 0) else M << -sh
        elif sh > mbits:
            continue
        else:
            a, rem, half = M >> sh, M & ((1 << sh) - 1), 1 << (sh - 1)
            if rem == half:
                i0 += a + ((o0 + a) & 1)
                i1 += a + ((o1 + a) & 1)
                o0 = o1 = 0
                continue
            c = a + (rem > half)
        i0 += c
        i1 += c
        o0 ^= c & 1
        o1 ^= c & 1
    return (min(i0, SAT), min(i1, SAT), o0, o1, E)


def compose(F, G):
    if F is INVALID or G is INVALID:
        return INVALID
    if F[4] == "any":
        E = G[4]
    elif G[4] == "any" or G[4] == F[4]:
        E = F[4]
    else:
        return INVALID
    g = (G[0], G[1])
    go = (G[2], G[3])
    return (sat(F[0] + g[F[2]]), sat(F[1] + g[F[3]]), go[F[2]], go[F[3]], E)


def apply(F, s):
    """New s, or None when F does not hold at s."""
    if F is INVALID:
        return None
    if F[4] == "any":
        return s
    u, E = units(s)
    if E != F[4]:
        return None
    nu = sat(u + (F[1] if u & 1 else F[0]))
    return None if nu > TWO53 else from_units(nu, E)


def mk(x):
    """x (a positive double) as M * 2^k."""
    if x == 0:
        return 0, 0
    m, e = math.frexp(x)
    M = int(math.ldexp(m, 53))
    k = e - 53
    while M and M % 2 == 0:
        M //= 2
        k += 1
    return M, k


def predict(P, A, margin):
    lo, hi = P * (1 - margin), (P + A) * (1 + margin)
    if not lo > 0:
        return None
    e0, e1 = binade(lo), binade(hi)
    return e0 if e0 == e1 else None


def ordered_sum(xs, chunk, fan, margin):
    """The GPU's method on the sequence xs (doubles >= 0, 0 = skipped)."""
    n = len(xs)
    nch = (n + chunk - 1) // chunk
    terms = [mk(x) for x in xs]
    csum = [math.fsum(xs[c * chunk:(c + 1) * chunk]) for c in range(nch)]
    pref = np.concatenate([[0.0], np.cumsum(csum)])
    level0 = []
    for c in range(nch):
        seg = terms[c * chunk:(c + 1) * chunk]
        if not any(M for M, _ in seg):
            level0.append(IDENT)
            continue
        E = predict(pref[c], csum[c], margin)
        if E is None:
            level0.append(INVALID)
            continue
        level0.append(acc_chunk(seg, E, 53))
    levels = [level0]
    while len(levels) < 2 or len(levels[-1]) > 1:
        prev = levels[-1]
        nxt = []
        for b in range(0, len(prev), fan):
            f = IDENT
            for g in prev[b:b + fan]:
                f = compose(f, g)
            nxt.append(f)
        levels.append(nxt)

    def replay(c, s):
        for x in xs[c * chunk:(c + 1) * chunk]:
            if x:
                s = s + x  # one IEEE f64 rounding, as the reference adds
        return s

    s, c, stats = 0.0, 0, {"replays": 0, "runs": 0}
    while c < nch:
        moved = False
        for L in range(len(levels) - 1, -1, -1):
            span = fan ** L
            if c % span:
                continue
            q = c // span
            lim = min(((q // fan) + 1) * fan if L + 1 < len(levels) else len(levels[L]), len(levels[L]))
            E = binade(s) if s else None
            t = 0
            # before the first value only empty runs; after it, runs in s's binade
            while q + t < lim and t < fan and levels[L][q + t] is not INVALID and \
                    levels[L][q + t][4] in (("any",) if E is None else ("any", E)):
                t += 1
            if t == 0:
                continue
            if E is None:
                c, moved = min((q + t) * span, nch), True
                break
            f = IDENT
            for g in levels[L][q:q + t]:
                f = compose(f, g)
            s2 = apply(f, s)
            if s2 is not None:
                s, c, moved = s2, min((q + t) * span, nch), True
                stats["runs"] += 1
                break
            if t > 1:
                s2 = apply(levels[L][q], s)
                if s2 is not None:
                    s, c, moved = s2, min((q + 1) * span, nch), True
                    break
        if not moved:
            s = replay(c, s)
            stats["replays"] += 1
            c += 1
    return s, stats


def sequential(xs):
    s = 0.0
    for x in xs:
        if x:
            s += x
    return s


def f32_terms(raw, scale):
    """The reference's values: (raw * scale_f32) as f64, and their squares."""
    raw = np.asarray(raw, np.float32)
    keep = np.isfinite(raw) & (raw > 0)
    v = np.where(keep, raw * np.float32(scale), np.float32(0)).astype(np.float64)
    return [float(x) for x in v], [float(x) * float(x) for x in v]


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("chunk,fan", [(4, 2), (8, 4), (16, 32)])
def test_map_like_sums_match_sequential(seed, chunk, fan):
    rng = np.random.default_rng(seed)
    n = 3000
    raw = (2.0 * np.sqrt(rng.integers(1, 3000, size=n))).astype(np.float32)
    raw[rng.random(n) < 0.3] = 0
    raw[rng.random(n) < 0.01] = -1.0
    for scale in (19.5, 8.0, 1e-30, 3.7e20):
        xs, qs = f32_terms(raw, scale)
        for seq in (xs, qs):
            got, _ = ordered_sum(seq, chunk, fan, 2.0 ** -20)
            assert got == sequential(seq)


@pytest.mark.parametrize("seed", range(8))
def test_ties_and_lost_values(seed):
    """A huge first value and then values at, above and below half an ulp of
    the running sum: round-half-even decided by the sum's parity at every
    step, and values that vanish."""
    rnd = random.Random(seed)
    xs = [2.0 ** 60]
    for _ in range(4000):
        r = rnd.random()
        if r < 0.5:
            xs.append(float((2 * rnd.randrange(1, 1 << 20) + 1) << 7))  # odd multiple of U/2 = 2^7
        elif r < 0.7:
            xs.append(float(rnd.randrange(1, 1 << 7)))                   # below U/2: lost
        elif r < 0.8:
            xs.append(0.0)
        else:
            xs.append(float(rnd.randrange(1, 1 << 40)))
    for chunk, fan in ((4, 2), (16, 4), (64, 32)):
        got, _ = ordered_sum(xs, chunk, fan, 2.0 ** -20)
        assert got == sequential(xs)


@pytest.mark.parametrize("margin", [2.0 ** -20, 2.0 ** -60, 0.0, 0.5])
def test_predictions_only_cost_time(margin):
    """Margins far too small (wrong predictions) or far too large (no
    predictions) give the same sum: the walker checks every step."""
    rng = np.random.default_rng(5)
    xs = [float(x) for x in rng.random(5000) * 1e3]
    got, _ = ordered_sum(xs, 8, 4, margin)
    assert got == sequential(xs)


def test_crossings_use_runs():
    """Between binade crossings the walker applies aggregated runs."""
    rng = np.random.default_rng(9)
    xs = [float(x) for x in rng.random(20000) * 100 + 1]
    got, st = ordered_sum(xs, 16, 8, 2.0 ** -20)
    assert got == sequential(xs)
    nch = (len(xs) + 15) // 16
    assert st["replays"] < nch // 10 and st["runs"] > 0


def test_leading_empty_chunks_are_skipped():
    """Empty chunks before the first value (outside the ROI) are skipped as runs."""
    xs = [0.0] * 5000 + [float(v) for v in np.random.default_rng(1).random(3000) * 50]
    got, st = ordered_sum(xs, 16, 8, 2.0 ** -20)
    assert got == sequential(xs) and st["replays"] < 20


@pytest.mark.parametrize("seed", range(5))
def test_thread_fold_equals_composition(seed):
    """The one-thread fold of a chunk equals the composition of its element
    functions, for sums of values (24-bit mantissas) and of squares (48-bit)."""
    rnd = random.Random(seed)
    for mbits in (24, 48):
        for _ in range(200):
            E = rnd.randrange(-20, 60)
            terms = []
            for _ in range(rnd.randrange(1, 40)):
                M = rnd.randrange(1, 1 << mbits)
                k = E - 52 + rnd.randrange(-8, mbits + 4)
                terms.append((M, k))
            f = IDENT
            for M, k in terms:
                f = compose(f, elem_fn(M, k, E))
            g = acc_chunk(terms, E, mbits)
            assert (min(f[0], SAT), min(f[1], SAT), f[2], f[3]) == g[:4]


def replay_units(xs, s):
    """The GPU replay (ordered.cu replay_chunk): s kept as a count of its
    binade's ulps, each value's rounded increment added with round half to
    even on that count, f64 addition only for the first value and for values
    that leave the binade."""
    in_units = s > 0 and math.isfinite(s)
    u, E = units(s) if in_units else (0, 0)
    for x in xs:
        if x == 0:
            continue
        M, k = mk(x)
        if in_units:
            sh = (E - 52) - k
            fits, tie, a = True, False, 0
            if sh <= 0:
                fits = sh > -54 and (M >> (54 + sh)) == 0
                a = M << -sh if fits else 0
            elif sh < 64:
                rem, half = M & ((1 << sh) - 1), 1 << (sh - 1)
                a = (M >> sh) + (rem > half)
                tie = rem == half
            if fits and u + a < TWO53:
                u += a + ((u + a) & 1) if tie else a
                if u == TWO53:
                    u, E = 1 << 52, E + 1
                continue
            s = from_units(u, E)
        s = s + x
        in_units = s > 0 and math.isfinite(s)
        if in_units:
            u, E = units(s)
    return from_units(u, E) if in_units else s


@pytest.mark.parametrize("seed", range(10))
def test_integer_replay_matches_sequential(seed):
    rnd = random.Random(seed)
    for _ in range(30):
        xs = []
        start = rnd.choice([0.0, 2.0 ** rnd.randrange(-40, 80)])
        for _ in range(rnd.randrange(1, 300)):
            r = rnd.random()
            if r < 0.3:
                xs.append(float((2 * rnd.randrange(1, 1 << 20) + 1)) * 2.0 ** rnd.randrange(-30, 30))
            elif r < 0.5:
                xs.append(0.0)
            elif r < 0.7:
                xs.append(rnd.random() * 2.0 ** rnd.randrange(-60, 70))
            else:
                xs.append(float(rnd.randrange(1, 1 << 24)) * 2.0 ** rnd.randrange(-20, 20))
        ref = start
        for x in xs:
            if x:
                ref = ref + x
        assert replay_units(xs, start) == ref
