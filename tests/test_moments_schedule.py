"""Work layout of the tensor-core moments kernel (CPU): a unit whose radial
bin carries orders l <= LM lays its (l, m) steps out as octets of orders
m = 8o .. 8o + 7 (octet o takes LM + 1 - 8o steps; step d holds l = m + d),
cuts them evenly over 4 P producer slots of at most 48 steps (24 accumulator
tiles of two steps), P CTAs per unit.  Every (l, m) with m <= l <= LM must be
produced by exactly one (slot, step, row), for every order the fill plans
(l <= 175).  This restates the device arithmetic (tc_octet_first, tc_steps,
tc_parts in dpx_internal.h; the slot bounds and tc_decode in hm_moments_tc).
"""

SLOT_STEPS = 48
TILES = 24


def octet_first(LM, o):
    return o * (LM + 1) - 4 * o * (o - 1)


def steps(LM):
    return octet_first(LM, LM // 8 + 1)


def parts(LM):
    return (steps(LM) + 4 * SLOT_STEPS - 1) // (4 * SLOT_STEPS)


def decode(LM, gs):
    O = LM // 8 + 1
    o = 0
    while o + 1 < O and octet_first(LM, o + 1) <= gs:
        o += 1
    return o, gs - octet_first(LM, o)


def test_every_order_pair_once():
    for LM in range(0, 176):
        S, P = steps(LM), parts(LM)
        W = 4 * P
        assert S == sum(LM + 1 - 8 * o for o in range(LM // 8 + 1))
        T = ((S + W - 1) // W + 1) // 2
        assert 1 <= T <= TILES
        seen = {}
        for sid in range(W):
            g0, g1 = sid * S // W, (sid + 1) * S // W
            assert 0 <= g1 - g0 <= SLOT_STEPS and g1 - g0 <= 2 * T
            for gs in range(g0, g1):
                o, d = decode(LM, gs)
                assert 0 <= d < LM + 1 - 8 * o
                for g in range(8):
                    m, l = 8 * o + g, 8 * o + g + d
                    if m <= LM and l <= LM:
                        assert (l, m) not in seen, (LM, l, m)
                        seen[(l, m)] = sid
        assert len(seen) == (LM + 1) * (LM + 2) // 2, LM


def test_parts_of_the_bench_orders():
    """Bins of the 20k-atom subunit at q_max 7.5 (l_b 57..64) take two CTAs a
    unit; low orders one."""
    assert [parts(LM) for LM in (10, 40, 47)] == [1, 1, 1]
    assert all(parts(LM) == 2 for LM in range(57, 65))
