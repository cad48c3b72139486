"""Dead-end pruning (the reference's reduce verb) in the oracle, on hand-built
contact graphs: a cycle with dangling chains, an electrode-fed path, isolated
rods and a chain that only peels over several passes."""
import numpy as np

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE


def graph(edges):
    I = np.array([e[0] for e in edges], np.uint32)
    J = np.array([e[1] for e in edges], np.uint32)
    return dict(I=I, J=J)


def test_cycle_with_dangling_chain(oracle):
    # 0-1-2-0 cycle, 3-4-5 chain hanging off 2, 6 isolated
    ct = graph([(0, 1), (1, 2), (0, 2), (2, 3), (3, 4), (4, 5)])
    keep, rounds = oracle.prune(7, ct)
    assert keep.tolist() == [True, True, True, False, False, False, False]
    assert rounds == 3  # 5 and 6, then 4, then 3


def test_electrodes_count_and_stay(oracle):
    # source - 0 - 1 - 2 - sink: every rod has two contacts; 3 hangs off the sink
    ct = graph([(0, SRC), (0, 1), (1, 2), (2, SNK), (3, SNK)])
    keep, rounds = oracle.prune(4, ct)
    assert keep.tolist() == [True, True, True, False] and rounds == 1
    # cut the sink contact: the whole path peels from the open end
    keep, rounds = oracle.prune(3, graph([(0, SRC), (0, 1), (1, 2)]))
    assert not keep.any() and rounds == 3


def test_duplicate_contacts_and_threshold(oracle):
    # two contacts between the same pair (two periodic images) count twice
    ct = graph([(0, 1), (0, 1)])
    keep, _ = oracle.prune(2, ct)
    assert keep.all()
    keep, _ = oracle.prune(2, ct, min_contacts=3)
    assert not keep.any()
    keep, rounds = oracle.prune(2, ct, min_contacts=0)
    assert keep.all() and rounds == 0
