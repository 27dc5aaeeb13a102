"""The wavefront order of the host-vector LSRK45 step (ew_lsrk45_step_host,
exwave_gb300/csrc/ew_api.cu), checked on the host against the sequential
step it must reproduce.

The step's five stages run chunk by chunk on one stream: stage s of chunk k
on diagonal d = k + 2 s, the stages of a diagonal from the last to the first.
Each stage reads its input register on the chunk and its two neighbours,
reads its accumulator on the chunk, and writes its output registers on the
chunk (the register tables of lsrk45_plan for the FP64 path and for the
reduced-precision paths).  The order is correct when every pair of stage
chunks that the sequential step orders through a register (read after
write, write after read, write after write) keeps its order, and when chunk
k of the state register is released only after every stage chunk that
touches it (the release follows the last such stage on chunk k + 1)."""
import itertools

import pytest

# (input X: read on chunks k-1..k+1, accumulator A: read on k, outputs: written on k)
PLANS = {
    # three FP64 registers N (the state in), T, P (the new state)
    "fp64": [("N", "N", ("T", "P")), ("T", "P", ("P", "N")), ("P", "N", ("N", "T")),
             ("N", "T", ("T", "P")), ("T", "P", ("P",))],
    # reduced precision: state S (in, split in place), accumulator P in
    # place, stage inputs X0 / X1
    "mixed": [("S", "S", ("X0", "P")), ("X0", "P", ("X1", "P")), ("X1", "P", ("X0", "P")),
              ("X0", "P", ("X1", "P")), ("X1", "P", ("P",))],
}
STATE = {"fp64": "N", "mixed": "S"}


def wave_order(K, lag=2):
    order = []
    for d in range(K + 4 * lag):
        for s in range(4, -1, -1):
            k = d - lag * s
            if 0 <= k < K:
                order.append((s, k))
    return order


def accesses(plan, s, k, K):
    x, a, outs = plan[s]
    reads = {(x, j) for j in range(max(0, k - 1), min(K, k + 2))} | {(a, k)}
    writes = {(r, k) for r in outs}
    return reads, writes


@pytest.mark.parametrize("name", sorted(PLANS))
@pytest.mark.parametrize("K", [1, 2, 3, 5, 16])
def test_wavefront_keeps_every_dependence(name, K):
    plan = PLANS[name]
    order = wave_order(K)
    assert sorted(order) == sorted(itertools.product(range(5), range(K)))
    pos = {op: i for i, op in enumerate(order)}
    acc = {op: accesses(plan, op[0], op[1], K) for op in order}
    for (s1, k1), (s2, k2) in itertools.permutations(order, 2):
        if s1 >= s2:
            continue  # the sequential step runs stage s1 before stage s2
        r1, w1 = acc[(s1, k1)]
        r2, w2 = acc[(s2, k2)]
        if (w1 & r2) or (r1 & w2) or (w1 & w2):
            assert pos[(s1, k1)] < pos[(s2, k2)], (name, (s1, k1), (s2, k2))


@pytest.mark.parametrize("name", sorted(PLANS))
@pytest.mark.parametrize("K", [1, 2, 16])
def test_state_chunks_released_after_their_last_use(name, K):
    plan = PLANS[name]
    state = STATE[name]
    order = wave_order(K)
    pos = {op: i for i, op in enumerate(order)}
    last = max(s for s in range(5) if state in (plan[s][0], plan[s][1]) + plan[s][2])
    for k in range(K):
        # released right after the last stage touching the state, on chunk k + 1
        rel = pos[(last, min(k + 1, K - 1))]
        for op in order:
            reads, writes = accesses(plan, op[0], op[1], K)
            if (state, k) in reads | writes:
                assert pos[op] <= rel, (name, k, op)


def test_a_lag_of_one_would_break_the_order():
    """With one diagonal per stage, a stage on chunk k and the previous
    stage on chunk k + 1 share a diagonal, and the descending order within
    it runs the later stage first: the check above must catch that."""
    plan, K = PLANS["fp64"], 6
    order = wave_order(K, lag=1)
    pos = {op: i for i, op in enumerate(order)}
    broken = False
    for (s1, k1), (s2, k2) in itertools.permutations(order, 2):
        if s1 < s2:
            r1, w1 = accesses(plan, s1, k1, K)
            r2, w2 = accesses(plan, s2, k2, K)
            if ((w1 & r2) or (r1 & w2) or (w1 & w2)) and pos[(s1, k1)] > pos[(s2, k2)]:
                broken = True
    assert broken
