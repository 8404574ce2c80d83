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
import dataclasses

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
        self.patterns = [(np.asarray(p), np.asarray(r)) for p, r in patterns]
        self.orders = list(orders) if orders is not None else [None] * len(patterns)
        self.options = options
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
    """Numeric factors of a batch on the GPU.

    With FP32 factors (precision PRECISION_MIXED) the FP64 fallback is per
    matrix: the batch handle refines every matrix's solution in FP64 and
    reports each matrix's backward error (row groups); the matrices that
    miss the target (too ill-conditioned for FP32 factors) are factored
    again in FP64 as a sub-batch of their own and their solutions replaced,
    instead of refactoring the whole batch in FP64.  The sub-batch's
    analyse is kept per set of matrices; its factors are redone after each
    refactorisation of the batch."""

    def __init__(self, bakeep, vals, options=None):
        self.bak = bakeep
        self.options = options or ssids.Options()
        self.mixed = self.options.precision == ssids.PRECISION_MIXED
        opts = self.options
        if self.mixed:
            opts = dataclasses.replace(self.options, fp64_fallback=False)
        self.vals = [np.asarray(v, dtype=np.float64) for v in vals]
        self.fk = ssids.Fkeep(bakeep.akeep, bakeep.stack_values(self.vals), opts)
        # refinement judges the backward error matrix by matrix (each with its
        # own norms), so every matrix of the batch meets the target
        from . import _native
        fl = _native.lib().spral_ssids_gpu_set_row_groups(
            self.fk.sym, bakeep.nmat, bakeep.mat_of_pivot.ctypes.data_as(ctypes.c_void_p))
        if fl != 0:
            raise RuntimeError(f"spral_gb300: row groups rejected, flag {fl}")
        self._subs = {}        # failing set -> [BatchAkeep, BatchFkeep or None, index map]
        self._sub_fresh = set()  # failing sets whose FP64 factors match the current values
        self.failed = np.zeros(0, dtype=np.int64)  # matrices of the last solve's FP64 fallback
        self.fallback_matrices = 0  # matrices refactored in FP64 since construction

    @property
    def inform(self):
        return self.fk.inform

    def refactor(self, vals):
        """Same-pattern refactorisation of every matrix of the batch (one
        captured-graph replay when no pivot was delayed last time)."""
        self.vals = [np.asarray(v, dtype=np.float64) for v in vals]
        self._sub_fresh.clear()
        return self.fk.refactor(self.bak.stack_values(self.vals))

    def refactor_dev(self, val_dev_ptr):
        """refactor() from the stacked values already on the device (their
        host copies, needed by a per-matrix fallback, are the last given)."""
        self._sub_fresh.clear()
        return self.fk.refactor_dev(val_dev_ptr)

    def group_errors(self):
        """Each matrix's scaled backward error after the last refined solve."""
        from . import _native
        out = np.zeros(self.bak.nmat)
        fl = _native.lib().spral_ssids_gpu_group_bwd_errors(
            self.fk.num, out.ctypes.data_as(ctypes.c_void_p), self.bak.nmat)
        if fl != 0:
            raise RuntimeError(f"spral_gb300: group backward errors unavailable, flag {fl}")
        return out

    def _fp64_sub(self, failed):
        """The FP64 sub-batch of the matrices `failed`, factored with their
        current values, and the map from its pivot positions to the batch's:
        [BatchAkeep, BatchFkeep, index map, (its device copy, once used)]."""
        key = tuple(int(i) for i in failed)
        ent = self._subs.get(key)
        if ent is None:
            pats = [self.bak.patterns[i] for i in key]
            ords = [self.bak.orders[i] for i in key]
            sub_ak = BatchAkeep(pats, ords, self.bak.options)
            idx = np.empty(sub_ak.n, dtype=np.int64)
            for j, i in enumerate(key):
                v = np.arange(self.bak.var_off[i + 1] - self.bak.var_off[i])
                idx[sub_ak.akeep.invp[sub_ak.var_off[j] + v]] = \
                    self.bak.akeep.invp[self.bak.var_off[i] + v]
            ent = [sub_ak, None, idx]
            self._subs[key] = ent
        sub_vals = [self.vals[i] for i in key]
        if ent[1] is None:
            ent[1] = BatchFkeep(ent[0], sub_vals,
                                dataclasses.replace(self.options,
                                                    precision=ssids.PRECISION_FP64))
            self.fallback_matrices += len(key)
        elif key not in self._sub_fresh:
            ent[1].refactor(sub_vals)
            self.fallback_matrices += len(key)
        self._sub_fresh.add(key)
        return ent

    def _failed_after_refinement(self):
        if not self.mixed:
            return np.zeros(0, dtype=np.int64)
        return np.nonzero(self.group_errors() > self.options.refine_tol)[0]

    def inertia(self):
        """(nmat, 3) array: negative eigenvalues, 2x2 pivots and zero pivots
        of each matrix (from the FP64 factors of the matrices the last
        refined solve refactored in FP64)."""
        per_node = self.fk.node_inertia()
        out = np.zeros((self.bak.nmat, 3), dtype=np.int64)
        np.add.at(out, self.bak.mat_of_node, per_node)
        key = tuple(int(i) for i in self.failed)
        if key and key in self._subs and self._subs[key][1] is not None:
            out[list(key)] = self._subs[key][1].inertia()
        return out

    def solve(self, bs):
        """Solve every matrix's system; bs[i] is n_i or n_i x nrhs (the same
        nrhs for all matrices)."""
        B, two = self.bak.stack_rhs(bs)
        return self.bak.split(self.fk.solve(B), two)

    def solve_refined(self, bs):
        """Solve with FP64 iterative refinement of the whole batch against its
        FP64 values (options max_refine / refine_tol), until every matrix's
        scaled backward error meets the target (FP32 factors: the matrices
        that cannot are solved again with FP64 factors of their own)."""
        B, two = self.bak.stack_rhs(bs)
        X = self.fk.solve_refined(B)
        self.failed = self._failed_after_refinement()
        if self.failed.size:
            sub_ak, sub = self._fp64_sub(self.failed)[:2]
            xs = sub.solve_refined([B[self.bak.var_off[i]:self.bak.var_off[i + 1]]
                                    for i in self.failed])
            for j, i in enumerate(self.failed):
                X[self.bak.var_off[i]:self.bak.var_off[i + 1]] = xs[j]
        return self.bak.split(X, two)

    def solve_refined_dev(self, b_dev, x_dev, nrhs=1):
        """solve_refined on device arrays in the batch's pivot order (torch
        CUDA tensors, n x nrhs column-major as nrhs contiguous vectors of n)."""
        import torch
        from . import _native
        L = _native.lib()
        n = self.bak.n
        it = ctypes.c_int(0)
        bw = ctypes.c_double(0)
        L.spral_ssids_gpu_solve_refined_dev(self.fk.num, nrhs, ctypes.c_void_p(b_dev.data_ptr()),
                                            ctypes.c_void_p(x_dev.data_ptr()), n,
                                            ctypes.byref(it), ctypes.byref(bw))
        self.failed = self._failed_after_refinement()
        if self.failed.size:
            ent = self._fp64_sub(self.failed)
            sub_ak, sub, idx = ent[:3]
            # the index map on the device, kept with the sub-batch
            if len(ent) < 4 or ent[3].device != x_dev.device:
                ent[3:] = [torch.as_tensor(idx, device=x_dev.device)]
            ix = ent[3]
            bm, xm = b_dev.view(nrhs, n), x_dev.view(nrhs, n)
            bs = bm[:, ix].contiguous()
            xs = torch.empty_like(bs)
            L.spral_ssids_gpu_solve_refined_dev(sub.fk.num, nrhs, ctypes.c_void_p(bs.data_ptr()),
                                                ctypes.c_void_p(xs.data_ptr()), sub_ak.n,
                                                ctypes.byref(it), ctypes.byref(bw))
            xm[:, ix] = xs
        return it.value

    def free(self):
        for ent in self._subs.values():
            if ent[1] is not None:
                ent[1].free()
        self._subs.clear()
        self.fk.free()
