"""Partitioned assembly (par_fe_space_t / dof_import_t / par_scalar_array_t) on the device,
and the nearest-neighbour exchange for multi-process runs.

``PartitionedFESpace(space, (np0, np1, np2))`` splits a structured continuous space into box
parts the way the reference's parallel FE space does for its tasks and keeps every part on the
context's device: per-part dof_import (exchange lists, weights, local-to-global map),
subassembled systems (``assemble``), ``comm`` (subassembled -> assembled interface values) and
a partitioned Jacobi-PCG (``solve``).

``neighbours_exchange`` is the same exchange between processes that each hold one part
(``torch.distributed`` point-to-point: gloo on the host, NCCL on devices), with the semantics
of the reference's l1_neighbours_exchange as used by par_scalar_array_t%comm
(Sources/Lib/LinearAlgebra/Vector/par_scalar_array.f90:498-533).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fe import _ptr


class PartitionedFESpace:
    def __init__(self, space, num_parts_x_dir):
        self.space = space
        nparts = (C.c_int32 * 3)(*[int(v) for v in num_parts_x_dir])
        h = C.c_void_p()
        L.check(L.lib().fg_partition_create(space.h, nparts, C.byref(h)), "fg_partition_create")
        self.h = h
        i = L.PartitionInfo()
        L.check(L.lib().fg_partition_get_info(h, C.byref(i)), "fg_partition_get_info")
        self.info = {k: getattr(i, k) for k, _ in L.PartitionInfo._fields_}
        self.num_parts = self.info["num_parts"]
        self.num_local_dofs = self.info["num_local_dofs"]

    def dof_import(self, part_id):
        """dof_import_t of part part_id (1-based, reference conventions) plus l2g, cells and the
        part's offset in the concatenated local vectors."""
        sz = L.DofImportSizes()
        L.check(L.lib().fg_partition_get_dof_import_sizes(self.h, int(part_id), C.byref(sz)),
                "fg_partition_get_dof_import_sizes")
        a = {"l2g": np.zeros(sz.num_dofs, np.int32), "weight": np.zeros(sz.num_dofs),
             "list_rcv": np.zeros(sz.num_rcv, np.int32), "rcv_ptrs": np.zeros(sz.num_rcv + 1, np.int32),
             "unpack_idx": np.zeros(sz.num_unpack, np.int32), "list_snd": np.zeros(sz.num_snd, np.int32),
             "snd_ptrs": np.zeros(sz.num_snd + 1, np.int32), "pack_idx": np.zeros(sz.num_pack, np.int32),
             "cells": np.zeros(sz.num_cells, np.int64)}
        L.check(L.lib().fg_partition_get_dof_import(self.h, int(part_id), *[_ptr(a[k]) for k in (
            "l2g", "weight", "list_rcv", "rcv_ptrs", "unpack_idx", "list_snd", "snd_ptrs", "pack_idx", "cells")]),
            "fg_partition_get_dof_import")
        a.update({"num_dofs": sz.num_dofs, "num_interior": sz.num_interior_dofs,
                  "num_interface": sz.num_interface_dofs, "first_local_dof": sz.first_local_dof})
        return a

    def assemble(self, integration):
        return PartitionedOperator(self, integration)

    def comm_device(self, x):
        """x (contiguous CUDA float64, num_local_dofs) <- comm(x), in place."""
        if not (x.is_cuda and x.is_contiguous() and x.numel() == self.num_local_dofs and x.dtype.itemsize == 8):
            raise ValueError("x must be a contiguous CUDA float64 tensor of num_local_dofs entries")
        L.check(L.lib().fg_partition_comm_device(self.h, _ptr(x)), "fg_partition_comm_device")
        return x

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_partition_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PartitionedOperator:
    """Subassembled systems of every part (par_fe_space_t's assembler), block diagonal over the
    concatenated local dofs; ``solve`` runs the partitioned Jacobi-PCG."""

    def __init__(self, pspace: PartitionedFESpace, integration):
        self.pspace = pspace
        g, keep = integration.to_c()
        h = C.c_void_p()
        L.check(L.lib().fg_partition_assemble(pspace.h, C.byref(g), C.byref(h)), "fg_partition_assemble")
        del keep
        self.h = h

    def get_matrix(self, symmetric_storage=True, one_based=True):
        n = self.pspace.num_local_dofs
        nnz = self.pspace.info["nnz_upper"] if symmetric_storage else self.pspace.info["nnz_full"]
        irp = np.zeros(n + 1, dtype=np.int64)
        ja = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        L.check(L.lib().fg_system_export_csr(self.h, int(symmetric_storage), int(one_based), _ptr(irp), _ptr(ja),
                                             _ptr(val)), "fg_system_export_csr")
        return irp, ja, val

    def get_translation(self):
        out = np.zeros(self.pspace.num_local_dofs)
        L.check(L.lib().fg_system_export_rhs(self.h, _ptr(out)), "fg_system_export_rhs")
        return out

    def solve(self, rtol=1e-8, atol=0.0, max_iters=100000, precond="jacobi"):
        p = L.SolverParams()
        L.lib().fg_solver_params_default(C.byref(p))
        p.precond = L.FG_PREC_JACOBI if precond == "jacobi" else L.FG_PREC_NONE
        p.rtol, p.atol, p.max_iters = rtol, atol, int(max_iters)
        x = np.zeros(self.pspace.space.num_free_dofs)
        info = L.SolveInfo()
        L.check(L.lib().fg_partition_solve(self.pspace.h, self.h, C.byref(p), _ptr(x), C.byref(info)),
                "fg_partition_solve")
        self.last_info = {k: getattr(info, k) for k, _ in L.SolveInfo._fields_}
        return x

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_system_destroy(self.h)
            self.h = None


def neighbours_exchange(dist, dof_import, x):
    """par_scalar_array_t%comm between processes: this rank holds one part (part id = rank + 1)
    with its dof_import (1-based lists) and its subassembled local vector x (torch tensor).
    Stage 1: non-owner interface values go to their owners, which add them in list_rcv order;
    stage 2: owners send the sums back and the other copies take them.  Returns x assembled."""
    import torch
    me = dist.get_rank() + 1

    def exchange(rcv_parts, rcv_ptrs, rcv_idx, snd_parts, snd_ptrs, snd_idx, add):
        reqs, bufs = [], []
        for k, q in enumerate(snd_parts):
            idx = torch.as_tensor(np.asarray(snd_idx[snd_ptrs[k] - 1:snd_ptrs[k + 1] - 1]) - 1, dtype=torch.long)
            buf = x[idx].clone()
            bufs.append(buf)
            reqs.append(dist.isend(buf, int(q) - 1))
        got = []
        for k, q in enumerate(rcv_parts):
            m = int(rcv_ptrs[k + 1] - rcv_ptrs[k])
            buf = torch.empty(m, dtype=x.dtype, device=x.device)
            dist.recv(buf, int(q) - 1)
            got.append(buf)
        for r in reqs:
            r.wait()
        for k, buf in enumerate(got):
            idx = np.asarray(rcv_idx[rcv_ptrs[k] - 1:rcv_ptrs[k + 1] - 1]) - 1
            for j, d in enumerate(idx):
                x[int(d)] = x[int(d)] + buf[j] if add else buf[j]

    di = dof_import
    assert me >= 1
    exchange(di["list_rcv"], di["rcv_ptrs"], di["unpack_idx"], di["list_snd"], di["snd_ptrs"], di["pack_idx"], True)
    exchange(di["list_snd"], di["snd_ptrs"], di["pack_idx"], di["list_rcv"], di["rcv_ptrs"], di["unpack_idx"], False)
    return x
