"""The staged-row slot mapping of the FP32/FP16/BF16 collide kernel's odd
A-A step, restated as index arithmetic on a small periodic lattice (the GPU
parity tests check the kernel's results bit for bit; this pins why it needs
no consumer barrier).

Odd step, x-row (y, z) of the kernel: the producer loads into staged row p
the populations of slot opp(p) of x-row (y - ey_p, z - ez_p) and afterwards
stores that staged row back where it was loaded from.  Consumer x reads its
incoming f_p at staged position x - ex_p of row p and writes its outgoing
f_q at position x + ex_q of row opp(q) (positions wrap: x periodic).  Then
  * every staged slot is read and written by one and the same consumer
    thread, so no thread overwrites a slot another has still to read;
  * every global population location is read and written once per step, by
    one x-row, so blocks working on different rows never touch the same
    location;
  * node n's outgoing f_q lands in slot q of node n + e_q and its incoming
    f_p comes from slot opp(p) of node n - e_p, the A-A odd step."""
import itertools

import numpy as np


def d3q19():
    e = [(0, 0, 0)]
    for a in range(3):
        for s in (1, -1):
            v = [0, 0, 0]
            v[a] = s
            e.append(tuple(v))
    for a, b in ((0, 1), (0, 2), (1, 2)):
        for sa, sb in itertools.product((1, -1), repeat=2):
            v = [0, 0, 0]
            v[a], v[b] = sa, sb
            e.append(tuple(v))
    return e


def d2q9():
    return [(0, 0, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, -1, 0), (1, 1, 0), (-1, 1, 0),
            (-1, -1, 0), (1, -1, 0)]


def opposite(e):
    return [e.index((-a, -b, -c)) for (a, b, c) in e]


def check_lattice(e, shape):
    Q = len(e)
    opp = opposite(e)
    S0, S1, S2 = shape
    reads = {}   # global (node, slot) -> x-rows that read it
    writes = {}
    for z in range(S2):
        for y in range(S1):
            row = (y, z)
            # staged row p: slot opp(p) of x-row (y - ey_p, z - ez_p)
            src = [((y - e[p][1]) % S1, (z - e[p][2]) % S2, opp[p]) for p in range(Q)]
            slot_reader = {}
            slot_writer = {}
            for x in range(S0):
                for p in range(Q):  # incoming f_p
                    i = (x - e[p][0]) % S0
                    assert (p, i) not in slot_reader
                    slot_reader[(p, i)] = x
                    yy, zz, sl = src[p]
                    node = (i, yy, zz)
                    # A-A odd step: incoming f_p of node n from slot opp(p) of n - e_p
                    assert node == ((x - e[p][0]) % S0, (y - e[p][1]) % S1, (z - e[p][2]) % S2)
                    assert sl == opp[p]
                    reads.setdefault((node, sl), []).append(row)
                for q in range(Q):  # outgoing f_q into staged row opp(q) at x + ex_q
                    r, i = opp[q], (x + e[q][0]) % S0
                    assert (r, i) not in slot_writer
                    slot_writer[(r, i)] = x
                    yy, zz, sl = src[r]  # stored back where staged row r came from
                    node = (i, yy, zz)
                    # A-A odd step: outgoing f_q of node n into slot q of n + e_q
                    assert node == ((x + e[q][0]) % S0, (y + e[q][1]) % S1, (z + e[q][2]) % S2)
                    assert sl == q
                    writes.setdefault((node, sl), []).append(row)
            # one thread per staged slot, reading and writing it
            assert slot_reader == slot_writer
            assert len(slot_reader) == Q * S0
    locations = S0 * S1 * S2 * Q
    assert len(reads) == len(writes) == locations
    for k, rows in reads.items():
        assert len(rows) == 1 and writes[k] == rows


def test_odd_step_slots_d3q19():
    check_lattice(d3q19(), (6, 5, 4))


def test_odd_step_slots_d2q9():
    check_lattice(d2q9(), (7, 5, 1))


def test_the_old_layout_needed_the_barrier():
    """Writing outgoing f_q into staged row q itself (at x + ex_q, stored to
    slot q of row y + e_q) lands on slots that other threads still read."""
    e = d3q19()
    Q, S0 = len(e), 6
    reader = {}
    for x in range(S0):
        for p in range(Q):
            reader[(p, (x - e[p][0]) % S0)] = x
    clashes = sum(reader[(q, (x + e[q][0]) % S0)] != x for x in range(S0) for q in range(Q))
    assert clashes == S0 * sum(1 for v in e if v[0] != 0)
    assert np.count_nonzero([v[0] for v in e]) == 10
