"""Decoder of the reference's partitioned-matrix ("signature") files.

TEST INFRASTRUCTURE ONLY (part of the oracle).  Reads rbParam.dat,
parParam.dat and nnzVal_<c>.dat as written by the reference's host
partitioner (Xilinx/HPC L2/sparse/src/sw/c++/gen_signature.cpp:44-77) and
returns every stored entry with its row, column, value, channel, partition and
position.  The layouts follow L2/sparse/include/sw/fp64/matrix_params.hpp:
RowBlockParam (329-471: 32-byte header, 8 x 32-byte blocks per row block),
ParParam (473-576: 32-byte header, 8 x 32-byte blocks per partition) and
NnzStore (578-688) as filled by Signature::gen_nnzStore
(signature.hpp:361-426): per channel, per row block, per partition, groups of
parEntries=4 values, with a 16 x uint16 row-index block every 512 entries
and a 16 x uint16 column-block block every 64 entries.  The decoding rule is
the reference's own Python twin (L2/sparse/tests/fp64/spmv/python/
matrix_params.py:300-323, signature.py:373-408).
"""
from __future__ import annotations

import os

import numpy as np

MEM_BYTES = 32
PAR_ENTRIES = 4
ACC_LATENCY = 8
CHANNELS = 16


def _u32(buf, off, cnt):
    return np.frombuffer(buf, np.uint32, cnt, off)


def _u16(buf, off, cnt):
    return np.frombuffer(buf, np.uint16, cnt, off)


def read_signature(path: str):
    with open(os.path.join(path, "rbParam.dat"), "rb") as f:
        rb = f.read()
    with open(os.path.join(path, "parParam.dat"), "rb") as f:
        par = f.read()
    nnz = []
    for c in range(CHANNELS):
        with open(os.path.join(path, "nnzVal_%d.dat" % c), "rb") as f:
            nnz.append(f.read())
    info = None
    ip = os.path.join(path, "info.dat")
    if os.path.exists(ip):
        info = np.fromfile(ip, np.int32, 6)
    return rb, par, nnz, info


def decode(path: str):
    """Returns a dict of arrays over all stored entries (padding included):
    row, col, val, channel, part (global partition id), pos (index within its
    channel chunk), plus 'info' (m, n, nnz, mPad, nPad, nnzPad)."""
    rb, par, nnz, info = read_signature(path)
    res = decode_bytes(rb, par, nnz)
    res["info"] = info
    return res


def decode_bytes(rb: bytes, par: bytes, nnz):
    """decode() over the rbParam, parParam and 16 nnzVal buffers in memory.
    Entries come in stream order: row block, then channel, then partition,
    then position in the channel chunk."""
    rb, par = bytes(rb), bytes(par)
    nnz = [bytes(b) for b in nnz]
    total_rows, total_rbs = _u32(rb, 0, 2)
    total_pars = int(_u32(par, 0, 1)[0])
    idx_width = MEM_BYTES // 2
    row_gap = PAR_ENTRIES * ACC_LATENCY
    row_mod = idx_width * row_gap
    col_mod = idx_width * PAR_ENTRIES
    out = {k: [] for k in ("row", "col", "val", "channel", "part", "pos")}
    offs = [MEM_BYTES] * CHANNELS
    s_par = 0
    for r in range(int(total_rbs)):
        base = MEM_BYTES + r * MEM_BYTES * 8
        s_row, _min_col, _ncols, npars = _u32(rb, base, 4)
        ch_row_off = _u16(rb, base + 2 * MEM_BYTES, CHANNELS)
        for c in range(CHANNELS):
            s_ch_row = int(s_row) + int(ch_row_off[c])
            off = offs[c]
            buf = nnz[c]
            for p in range(int(npars)):
                pid = s_par + p
                pbase = MEM_BYTES + pid * MEM_BYTES * 8
                ch_nnz = int(_u32(par, pbase + 2 * MEM_BYTES, CHANNELS)[c])
                s_par_col = int(_u32(par, pbase + 4 * MEM_BYTES, 1)[0])
                ch_col_off = int(_u16(par, pbase + 5 * MEM_BYTES, CHANNELS)[c])
                s_ch_col = s_par_col + ch_col_off
                row_idx = col_idx = None
                for i in range(0, ch_nnz, PAR_ENTRIES):
                    if i % row_mod == 0:
                        row_idx = _u16(buf, off, idx_width)
                        off += MEM_BYTES
                    if i % col_mod == 0:
                        col_idx = _u16(buf, off, idx_width)
                        off += MEM_BYTES
                    vals = np.frombuffer(buf, np.float64, PAR_ENTRIES, off)
                    off += MEM_BYTES
                    rr = int(row_idx[(i % row_mod) // row_gap]) + s_ch_row
                    cb = (int(col_idx[(i % col_mod) // PAR_ENTRIES]) + s_ch_col) * PAR_ENTRIES
                    for j in range(PAR_ENTRIES):
                        out["row"].append(rr)
                        out["col"].append(cb + j)
                        out["val"].append(vals[j])
                        out["channel"].append(c)
                        out["part"].append(pid)
                        out["pos"].append(i + j)
            offs[c] = off
        s_par += int(npars)
    assert s_par == total_pars
    res = {k: np.array(v) for k, v in out.items()}
    res["total_rows"] = int(total_rows)
    return res


def fpga_order_spmv(dec, x, rows: int):
    """y = A x (first `rows` rows) in the summation order the reference's FPGA
    SpMV spells out in its C source, over every stored entry of a decoded
    signature (padding included, stream order):

    - multAddX (L1/sparse/include/hw/xf_sparse/fp64/spmv.hpp:136-157): each
      group of 4 stored entries, the products v_j * x_j (each rounded) summed
      left to right from 0;
    - regAcc (spmv.hpp:159-185): each run of 8 group sums (the 32 entries under
      one row index) summed left to right from 0;
    - rowMemAcc (spmv.hpp:452-476): a row's run sums added to its row store,
      which starts at 0, in stream order (its row block's partitions in order);
    - accY (dataMovers.hpp:339-375): the 16 channels' values for the row summed
      from 0 in channel order; a row belongs to one channel and the others give
      +0, so y = 0 + (row store).

    Every operation is a separate IEEE double multiply or add (numpy
    elementwise), so the result is the C semantics of that source."""
    val = np.asarray(dec["val"], np.float64)
    col = np.asarray(dec["col"], np.int64)
    row = np.asarray(dec["row"], np.int64)
    xp = np.zeros(max(int(col.max()) + 1, len(x)), np.float64)
    xp[:len(x)] = x
    prod = val * xp[col]
    p4 = prod.reshape(-1, 4)
    grp = 0.0 + p4[:, 0]
    for j in range(1, 4):
        grp = grp + p4[:, j]
    g8 = grp.reshape(-1, 8)
    run = 0.0 + g8[:, 0]
    for j in range(1, 8):
        run = run + g8[:, j]
    run_row = row[::32]
    order = np.argsort(run_row, kind="stable")  # keeps stream order within a row
    rr, rv = run_row[order], run[order]
    first = np.searchsorted(rr, rr, side="left")
    k = np.arange(rr.size) - first  # position of the run within its row
    nrow = max(rows, int(run_row.max()) + 1)
    store = np.zeros(nrow, np.float64)
    for step in range(int(k.max()) + 1 if k.size else 0):
        m = k == step
        store[rr[m]] = store[rr[m]] + rv[m]
    return (0.0 + store)[:rows]


def fpga_order_spmv_literal(dec, x, rows: int):
    """fpga_order_spmv written as the plain loops of the reference source
    (small cases only; pins the vectorised form)."""
    val, col, row = dec["val"], dec["col"], dec["row"]
    store = {}
    for r0 in range(0, len(val), 32):
        run = 0.0
        for b in range(8):
            grp = 0.0
            for j in range(4):
                e = r0 + 4 * b + j
                xv = float(x[col[e]]) if col[e] < len(x) else 0.0
                grp += float(val[e]) * xv
            run += grp
        r = int(row[r0])
        store[r] = store.get(r, 0.0) + run
    return np.array([0.0 + store.get(i, 0.0) for i in range(rows)])


def stored_order(dec):
    """Non-padding entries (value != 0) of a decoded signature, ordered by
    (row, partition, position): the order in which the reference holds each
    row's entries."""
    keep = dec["val"] != 0
    row, part, pos = dec["row"][keep], dec["part"][keep], dec["pos"][keep]
    order = np.lexsort((pos, part, row))
    return {k: dec[k][keep][order] for k in ("row", "col", "val", "part")}


def transy_frame(start_addr: int, rows: int, y) -> bytes:
    """The dSpmv transY framing (dSpmv/hw/include/impl/transY.hpp:35-65) of
    the first `rows` values of y: one 64-byte word {start_addr, rows, 0...}
    (uint32 little endian), then the values packed eight per 64-byte word in
    arrival order, the last word zero-filled; the HLS loop always emits a final
    data word, so rows = 0 still yields one zero word."""
    head = np.zeros(16, np.uint32)
    head[0] = start_addr
    head[1] = rows
    words = max(1, (rows + 7) // 8)
    data = np.zeros(words * 8, np.float64)
    data[:rows] = np.asarray(y, np.float64)[:rows]
    return head.tobytes() + data.tobytes()
