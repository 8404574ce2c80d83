"""Host-side batch logic (no GPU): the block-diagonal forest and its maps."""
import numpy as np

from spral_gb300 import batch, matrices as M


def test_batch_forest_maps_nodes_to_matrices():
    sides = [8, 11, 8, 16]
    pats, orders = [], []
    for s in sides:
        p, r, _ = M.laplacian_2d(s, s, -0.5)
        pats.append((p, r))
        orders.append(M.nd_order_grid(s, s))
    bak = batch.BatchAkeep(pats, orders)
    assert bak.n == sum(s * s for s in sides)
    ak = bak.akeep
    # every node's pivots belong to one matrix, and every matrix owns
    # exactly its own number of pivots
    piv_mat = np.searchsorted(bak.var_off, ak.invp, side="right") - 1
    owned = np.zeros(len(sides), dtype=np.int64)
    for node in range(ak.nnodes):
        cols = piv_mat[ak.sptr[node] - 1:ak.sptr[node + 1] - 1]
        assert np.all(cols == bak.mat_of_node[node])
        owned[bak.mat_of_node[node]] += len(cols)
    assert list(owned) == [s * s for s in sides]
    # a forest: each matrix contributes at least one root
    roots = np.nonzero(ak.sparent[:ak.nnodes] > ak.nnodes)[0]
    assert set(bak.mat_of_node[roots]) == set(range(len(sides)))


def test_batch_stacking_and_split():
    pats = [(np.array([0, 1, 2]), np.array([0, 1])), (np.array([0, 2, 3]), np.array([0, 1, 1]))]
    bak = batch.BatchAkeep(pats)
    v = bak.stack_values([np.array([1.0, 2.0]), np.array([3.0, 4.0, 5.0])])
    assert v.tolist() == [1, 2, 3, 4, 5]
    B, two = bak.stack_rhs([np.ones(2), 2 * np.ones(2)])
    assert B.shape == (4, 1) and not two
    xs = bak.split(B, two)
    assert xs[1].tolist() == [2.0, 2.0]
