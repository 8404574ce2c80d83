"""Batched factorisation and solve of many independent sparse symmetric
matrices on one GPU.

The matrices are stacked block-diagonally, so their assembly trees form one
forest.  Every level set of every tree then goes through the same kernel
launches (each launch covers the level's fronts of the whole batch), a
same-pattern refactorisation of the batch replays one captured CUDA graph of
the whole level sweep, and one solve pass serves every matrix's right-hand
sides.  Results per matrix are identical to factoring the matrix alone: each
front is computed by the same kernels on the same data, whatever else shares
the launch.

The reference has no batched interface; a caller of the reference factors
the matrices one ssids_analyse/ssids_factor/ssids_solve sequence at a time.
"""
import ctypes

import numpy as np

from . import ssids


class BatchAkeep:
    """Analyse of a batch: the block-diagonal forest and the maps between
    matrices, variables and assembly-tree nodes."""

    def __init__(self, patterns, orders=None, options=None):
        """patterns: sequence of (ptr, row) lower-CSC patterns (0-based);
        orders: per-matrix pivot orders (order[i] = pivot position of
        variable i), or None for the minimum-degree ordering."""
        if len(patterns) == 0:
            raise ValueError("empty batch")
        sizes = np.array([len(p) - 1 for p, _ in patterns], dtype=np.int64)
        nnzs = np.array([int(p[-1]) for p, _ in patterns], dtype=np.int64)
        self.nmat = len(patterns)
        self.var_off = np.concatenate([[0], np.cumsum(sizes)])
        self.nz_off = np.concatenate([[0], np.cumsum(nnzs)])
        ptr = [np.zeros(1, dtype=np.int64)]
        row, order = [], []
        for i, (p, r) in enumerate(patterns):
            p = np.asarray(p, dtype=np.int64)
            ptr.append(p[1:] + self.nz_off[i])
            row.append(np.asarray(r, dtype=np.int64) + self.var_off[i])
            o = ssids.order_mindeg(p, r) if orders is None or orders[i] is None else orders[i]
            order.append(np.asarray(o, dtype=np.int64) + self.var_off[i])
        self.ptr = np.concatenate(ptr)
        self.row = np.concatenate(row).astype(np.int32)
        self.akeep = ssids.analyse(self.ptr, self.row, np.concatenate(order).astype(np.int32),
                                   options)
        mat_of_var = np.repeat(np.arange(self.nmat), sizes)
        first = self.akeep.invp[self.akeep.sptr[:-1] - 1]  # first pivot of each node
        self.mat_of_node = mat_of_var[first]
        # matrix of each pivot position: the refinement's row groups
        self.mat_of_pivot = np.ascontiguousarray(mat_of_var[self.akeep.invp], dtype=np.int32)

    @property
    def n(self):
        return int(self.var_off[-1])

    def stack_values(self, vals):
        vals = [np.asarray(v, dtype=np.float64) for v in vals]
        if len(vals) != self.nmat:
            raise ValueError("one value array per matrix")
        for i, v in enumerate(vals):
            if v.size != self.nz_off[i + 1] - self.nz_off[i]:
                raise ValueError(f"matrix {i}: value count does not match its pattern")
        return np.concatenate(vals)

    def stack_rhs(self, bs):
        bs = [np.asarray(b, dtype=np.float64) for b in bs]
        two = bs[0].ndim == 2
        return np.concatenate([b if two else b[:, None] for b in bs], axis=0), two

    def split(self, x, two=True):
        out = [x[self.var_off[i]:self.var_off[i + 1]] for i in range(self.nmat)]
        return out if two else [o[:, 0] for o in out]


class BatchFkeep:
    """Numeric factors of a batch on the GPU."""

    def __init__(self, bakeep, vals, options=None):
        self.bak = bakeep
        self.fk = ssids.Fkeep(bakeep.akeep, bakeep.stack_values(vals), options)
        # refinement judges the backward error matrix by matrix (each with its
        # own norms), so every matrix of the batch meets the target
        from . import _native
        fl = _native.lib().spral_ssids_gpu_set_row_groups(
            self.fk.sym, bakeep.nmat, bakeep.mat_of_pivot.ctypes.data_as(ctypes.c_void_p))
        if fl != 0:
            raise RuntimeError(f"spral_gb300: row groups rejected, flag {fl}")

    @property
    def inform(self):
        return self.fk.inform

    def refactor(self, vals):
        """Same-pattern refactorisation of every matrix of the batch (one
        captured-graph replay when no pivot was delayed last time)."""
        return self.fk.refactor(self.bak.stack_values(vals))

    def inertia(self):
        """(nmat, 3) array: negative eigenvalues, 2x2 pivots and zero pivots
        of each matrix."""
        per_node = self.fk.node_inertia()
        out = np.zeros((self.bak.nmat, 3), dtype=np.int64)
        np.add.at(out, self.bak.mat_of_node, per_node)
        return out

    def solve(self, bs):
        """Solve every matrix's system; bs[i] is n_i or n_i x nrhs (the same
        nrhs for all matrices)."""
        B, two = self.bak.stack_rhs(bs)
        return self.bak.split(self.fk.solve(B), two)

    def solve_refined(self, bs):
        """Solve with FP64 iterative refinement of the whole batch against its
        FP64 values (options max_refine / refine_tol), until every matrix's
        scaled backward error meets the target."""
        B, two = self.bak.stack_rhs(bs)
        return self.bak.split(self.fk.solve_refined(B), two)

    def free(self):
        self.fk.free()
