"""The mixed SDF kernel's expanded sphere test (csrc/sdf_sub.cu, exp_term / exp_g / exp_b /
exp_pass_reach) restated in FP32 with FMA and directed rounding emulated in extended
precision. Its two guarantees, checked on adversarial cases (cells anywhere in the
sub-brick, entries at the reach's boundary, bounds from zero up, sub-brick radii from
zero up):
- every entry within the scalar reach L = RU(b (1 + 20u) + term) of the cell passes;
- an entry that passes lies within exp_pass_reach of the cell (the warp pre-test's reach).
With the margins taken out (no widening of B and T), entries within L fail: the
margins are what makes the test safe."""
import numpy as np

F32 = np.float32
LD = np.longdouble
U = F32(2.0 ** -24)


def _rn(v):
    return F32(v)


def _ru(v):
    r = F32(v)
    if LD(r) < v:
        r = np.nextafter(r, F32(np.inf))
    return r


def _fma(a, b, c):
    return _rn(LD(a) * LD(b) + LD(c))


def _fma_ru(a, b, c):
    return _ru(LD(a) * LD(b) + LD(c))


def _mul_ru(a, b):
    return _ru(LD(a) * LD(b))


def _add_ru(a, b):
    return _ru(LD(a) + LD(b))


def _reach_term(w, r):
    return _fma_ru(w, F32(1 + 20 * U), _mul_ru(F32(17 * U), r))


def _expanded(p, c, b, term, r, widen=True):
    """(passes, exp_pass_reach) of the kernel's expanded test for cell p and entry c."""
    sr = _fma_ru(F32(0.002), r, F32(1e-18)) if widen else F32(0)
    t = _fma_ru(term, F32(1 + 51 * U), sr) if widen else term
    g = _fma(-t, t, _fma(c[0], c[0], _fma(c[1], c[1], _rn(LD(c[2]) * LD(c[2])))))
    cp = (c * F32(-2)).astype(np.float32)
    p2 = _fma(p[0], p[0], _fma(p[1], p[1], _rn(LD(p[2]) * LD(p[2]))))
    bb = _mul_ru(b, F32(1 + 71 * U)) if widen else _mul_ru(b, F32(1 + 20 * U))
    k = _fma(bb, bb, -p2)
    a = _fma(p[0], cp[0], _fma(p[1], cp[1], _fma(p[2], cp[2], _fma(F32(-2) * bb, t, g))))
    reach = _fma_ru(_add_ru(bb, t), F32(1 + 21 * U), _mul_ru(F32(0.0016), r))
    return a <= k, reach


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        r = F32(rng.choice([0.0, 0.5, 1.3, 2.6, 10.0]) * 10.0 ** rng.uniform(-6, 3))
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        p = (v * float(r) * rng.uniform(0, 1)).astype(np.float32)
        s = max(float(r), 1e-6)
        b = F32(10.0 ** rng.uniform(-8, 3) * rng.choice([0, 1, 1, 1]) * s)
        term = _reach_term(F32(10.0 ** rng.uniform(-8, 2) * s), r)
        L = LD(b) * LD(F32(1 + 20 * U)) + LD(term)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        scale = rng.choice([1 - 1e-6, 1 - 1e-7, 1.0, 1 + 1e-7, rng.uniform(0, 1.2)])
        c = (p.astype(np.float64) + d * float(L) * scale).astype(np.float32)
        d2 = sum((LD(p[i]) - LD(c[i])) ** 2 for i in range(3))
        yield p, c, b, term, r, L, d2


def test_expanded_test_admits_the_scalar_reach_and_stays_within_the_warp_reach():
    inside = misses = beyond = 0
    for p, c, b, term, r, L, d2 in _cases(20000, 5):
        ok, reach = _expanded(p, c, b, term, r)
        if d2 <= L * L:
            inside += 1
            misses += not ok
        if ok and d2 > LD(reach) ** 2:
            beyond += 1
    assert inside > 5000
    assert misses == 0
    assert beyond == 0


def test_without_the_margins_entries_within_the_reach_fail():
    misses = 0
    for p, c, b, term, r, L, d2 in _cases(4000, 6):
        ok, _ = _expanded(p, c, b, term, r, widen=False)
        misses += d2 <= L * L and not ok
    assert misses > 0
