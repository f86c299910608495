"""The static-scene traversal pushes children through a table instead of
walking the four child positions: for every ray octant, traversal code and
4-bit hit mask, the table must give the same child to descend into and the
same pushed children, in the same stack order, as the reference's
front-to-back walk (BVH4::traverse, src/accel/bvh4.rs:148-170, with
TRAVERSAL_TABLE from sub_crates/bvh_order/build.rs:5-100).  Host-side only."""
from psychopath_gb300 import gpu

NONE = None


def walk(order, count, m):
    """Reference order: positions 3..0 of the table entry; every hit child but
    the first in front-to-back order is pushed, deepest first."""
    m &= (1 << count) - 1
    nxt, pushed = NONE, []
    for i in range(3, -1, -1):
        ci = (order >> (2 * i)) & 3
        if (m >> ci) & 1:
            if nxt is not NONE:
                pushed.append(nxt)
            nxt = ci
    return nxt, pushed


def reference_order(rd, code):
    """Front-to-back child order of sub_crates/bvh_order/build.rs (restated)."""
    ray = [rd & 1, (rd >> 1) & 1, (rd >> 2) & 1]
    k = 0
    for s2 in range(3):
        for s1 in range(3):
            for s0 in range(3):
                p = [0, 1, 2, 3]
                if ray[s1]:
                    p[0], p[1] = p[1], p[0]
                if ray[s2]:
                    p[2], p[3] = p[3], p[2]
                if ray[s0]:
                    p[0], p[2] = p[2], p[0]
                    p[1], p[3] = p[3], p[1]
                if k == code:
                    return p
                k += 1
    for s1 in range(3):
        for s0 in range(3):
            p = [0, 1, 2]
            if ray[s1]:
                p[0], p[1] = p[1], p[0]
            if ray[s0]:
                p[0], p[1] = p[1], p[0]
                p[0], p[2] = p[2], p[0]
            if k == code:
                return p
            k += 1
    for s1 in range(3):
        for s0 in range(3):
            p = [0, 1, 2]
            if ray[s1]:
                p[1], p[2] = p[2], p[1]
            if ray[s0]:
                p[0], p[2] = p[2], p[0]
                p[0], p[1] = p[1], p[0]
            if k == code:
                return p
            k += 1
    for s0 in range(3):
        p = [0, 1]
        if ray[s0]:
            p[0], p[1] = p[1], p[0]
        if k == code:
            return p
        k += 1
    raise ValueError(code)


def test_device_table_orders_children_as_the_reference(gpu_lib):
    table, _, _ = gpu.push_tables()
    for rd in range(8):
        for code in range(48):
            p = reference_order(rd, code)
            got = [(int(table[rd, code]) >> (2 * i)) & 3 for i in range(4)]
            assert got[:len(p)] == p, (rd, code)
            # positions past the child count name the empty slots
            assert sorted(got) == [0, 1, 2, 3], (rd, code)


def test_push_table_matches_front_to_back_walk(gpu_lib):
    table, rows, lut = gpu.push_tables()
    assert rows.max() < 32
    for rd in range(8):
        for code in range(48):
            count = 4 if code < 27 else (3 if code < 45 else 2)
            for m in range(16):
                nxt, pushed = walk(int(table[rd, code]), count, m)
                e = int(lut[rows[rd, code], m])
                if nxt is NONE:
                    assert e & 0x800 == 0, (rd, code, m)
                    continue
                assert e & 0x800, (rd, code, m)
                n = (e >> 8) & 7
                got = [(e >> (2 + 2 * j)) & 3 for j in range(n)]
                assert (e & 3) == nxt and got == pushed, (rd, code, m, e)
