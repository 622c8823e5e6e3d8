"""Index maps of the FP64 global passes' subsystem-major workspace
(pcr_tile.cuh, capi.cpp), restated and checked on the CPU.

After s strides of PCR-Penta, the rows i = t*G + r (G = 2^s) of a system of
n rows form subsystem r, local row t.  A pass that starts at stride G and runs
K strides writes its output so that each subsystem of the next level
G2 = G*2^K is contiguous: subsystem r2 starts r2*(n/G2) + min(r2, n%G2) rows
into the system.  The next pass reads its subsystem r2 as one run from there.
These tests check that the writer's map (r, t) -> (r + (t mod 2^K)*G, t >> K)
puts global row i where the reader looks for it, that every slot of [0, n) is
written exactly once, and that loads stay inside their subsystem's run."""
import numpy as np
import pytest


def sub_off(n, g, r):
    return r * (n // g) + min(r, n % g)


def sub_rows(n, g, r):
    return (n - 1 - r) // g + 1


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 100, 257, 1000, 1025, 4099, 65536, 70001])
@pytest.mark.parametrize("G,K", [(1, 1), (1, 2), (1, 3), (4, 2), (16, 2), (8, 3), (2, 4), (64, 2)])
def test_writer_and_reader_maps_agree(n, G, K):
    G2 = G << K
    slot_of_row = np.full(n, -1, dtype=np.int64)
    hits = np.zeros(n, dtype=np.int64)
    # writer: every (subsystem r, local row t) of level G
    for r in range(min(G, n)):
        for t in range(sub_rows(n, G, r)):
            i = t * G + r
            r2 = r + (t & ((1 << K) - 1)) * G
            t2 = t >> K
            assert t2 * G2 + r2 == i
            assert 0 <= r2 < G2 and t2 < sub_rows(n, G2, r2)
            gi = sub_off(n, G2, r2) + t2
            assert 0 <= gi < n
            hits[gi] += 1
            slot_of_row[i] = gi
    assert (hits == 1).all()
    # reader at level G2: subsystem r2, local row t2 -> the slot the writer used
    for r2 in range(min(G2, n)):
        base = sub_off(n, G2, r2)
        for t2 in range(sub_rows(n, G2, r2)):
            assert slot_of_row[t2 * G2 + r2] == base + t2


@pytest.mark.parametrize("n", [5, 1000, 65536, 70001])
@pytest.mark.parametrize("g", [1, 2, 16, 256, 1024])
def test_subsystem_runs_tile_the_system(n, g):
    """The runs of the subsystems of one level are disjoint and cover [0, n)."""
    ends = 0
    for r in range(min(g, n)):
        assert sub_off(n, g, r) == ends
        ends += sub_rows(n, g, r)
    assert ends == n
