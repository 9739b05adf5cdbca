"""CPU restatement of the reference's partitioned-matrix ("signature") writer.

TEST INFRASTRUCTURE ONLY (part of the oracle): the checker of the device
exporter (xJPCG_gbExportSignature).  Nothing in hpc_gb300 imports it.

Restates Signature::gen_sig / update_sig of Xilinx/HPC
L2/sparse/include/sw/fp64/signature.hpp with the parameters SpmPar is built
with for xJPCG (parEntries 4, accLatency 8, 16 channels, 4096 x 4096
partitions, 256-bit words):

  gen_rbs          (signature.hpp:95-138)  row blocks: entries stably sorted
                   by row; a block starts at the first row not yet covered
                   and takes the rows below start + 4096.
  genPars4Rb       (:140-173)  column partitions of a block: entries stably
                   sorted by column; a partition starts at the first uncovered
                   column rounded down to 4 and takes the columns below
                   start + 4096.
  pad_par          (:186-231)  each partition stably sorted by row; per row,
                   its entries placed into aligned 4-column groups (a slot
                   whose column is absent is a padding entry), then the row
                   padded to a multiple of 32 slots.
  gen_chPars       (:250-316)  each padded partition cut into 16 channel
                   chunks of about nnz/16 slots, each cut moved forward to
                   the end of the row it falls in.
  update_rbParams  (:318-359), gen_nnzStore (:361-426), update_nnzStore
                   (:427-465) and the buffer layouts of RowBlockParam,
                   ParParam and NnzStore (matrix_params.hpp:329-688).

The loops are plain Python: for the small fixture matrices only.
"""
from __future__ import annotations

import numpy as np

PAR = 4          # parEntries
ACC = 8          # accLatency
CH = 16          # HBM channels
MAXR = 4096      # maxRows of a row block
MAXC = 4096      # maxCols of a partition
WORD = 32        # bytes per 256-bit word
PAD = -1         # source index of a padding slot (ZERO_VAL)


def _u32(words):
    return np.asarray(words, dtype=np.uint32).tobytes()


def _u16(vals):
    return (np.asarray(vals, dtype=np.int64) & 0xFFFF).astype(np.uint16).tobytes()


def _word(data: bytes) -> bytes:
    assert len(data) <= WORD
    return data + b"\0" * (WORD - len(data))


class Layout:
    """The structure of a partitioned matrix: everything but the values."""


def partition(m, n, row, col):
    """Structure of gen_sig for a COO matrix with 0-based indices (entry k is
    input position k).  Returns a Layout."""
    row = np.asarray(row, np.int64)
    col = np.asarray(col, np.int64)
    nnz = row.size
    L = Layout()
    L.m, L.n, L.nnz = int(m), int(n), int(nnz)
    by_row = np.argsort(row, kind="stable")
    rs = row[by_row]
    blocks = []      # (entry indices in row-sorted order)
    s = 0
    while s < nnz:
        e = int(np.searchsorted(rs, rs[s] + MAXR, "left"))
        blocks.append(by_row[s:e])
        s = e
    L.blocks = []
    L.parts = []     # padded partitions: dict(rows, cols, src, block)
    for b, ent in enumerate(blocks):
        br, bc = row[ent], col[ent]
        binfo = {"minRow": int(br.min()), "minCol": int(bc.min()), "m": int(br.max() - br.min() + 1),
                 "n": int(bc.max() - bc.min() + 1), "nnz": int(ent.size), "firstPart": len(L.parts)}
        by_col = ent[np.argsort(bc, kind="stable")]
        cs = col[by_col]
        s = 0
        start = (int(cs[0]) // PAR) * PAR
        while s < by_col.size:
            e = int(np.searchsorted(cs, start + MAXC, "left"))
            pent = by_col[s:e]
            L.parts.append(_pad(pent[np.argsort(row[pent], kind="stable")], row, col, b))
            s = e
            if s < by_col.size:
                start = (int(cs[s]) // PAR) * PAR
        binfo["numPars"] = len(L.parts) - binfo["firstPart"]
        L.blocks.append(binfo)
    for p in L.parts:
        _channels(p)
    return L


def _pad(ent, row, col, block):
    """pad_par: per row, aligned groups of PAR slots, rows padded to PAR*ACC."""
    prow, pcol, psrc = [], [], []
    i = 0
    while i < ent.size:
        r = row[ent[i]]
        j = i
        while j < ent.size and row[ent[j]] == r:
            j += 1
        mod, base, count = 0, (int(col[ent[i]]) // PAR) * PAR, 0
        k = i
        while k < j:
            c = int(col[ent[k]])
            if mod == 0:
                base = (c // PAR) * PAR
            prow.append(r)
            if c != base + mod:
                pcol.append(base + mod)
                psrc.append(PAD)
            else:
                pcol.append(c)
                psrc.append(int(ent[k]))
                k += 1
            count += 1
            mod = (mod + 1) % PAR
        while count % (PAR * ACC):
            prow.append(r)
            pcol.append(base + mod)
            psrc.append(PAD)
            mod = (mod + 1) % PAR
            count += 1
        i = j
    return {"rows": np.array(prow, np.int64), "cols": np.array(pcol, np.int64), "src": np.array(psrc, np.int64),
            "block": block}


def _extent(v):
    return (int(v.min()), int(v.max() - v.min() + 1)) if v.size else (0, 0)


def _channels(p):
    """gen_chPars: 16 chunks cut at row boundaries."""
    rows, cols = p["rows"], p["cols"]
    nnz = rows.size
    per = nnz // CH
    p["minCol"], p["ncols"] = _extent(cols)
    p["minRow"], p["nrows"] = _extent(rows)
    chunks = []
    s = 0
    for c in range(CH):
        e = nnz if (c == CH - 1 or s + per >= nnz) else s + per
        while 0 < e < nnz and rows[e] == rows[e - 1]:
            e += 1
        minRow, m = _extent(rows[s:e])
        minCol, ncol = _extent(cols[s:e])
        chunks.append({"s": s, "e": e, "minRow": minRow, "m": m, "minCol": minCol, "n": ncol})
        s = e
    p["chunks"] = chunks


def rb_param(L) -> bytes:
    out = [_word(_u32([L.m, len(L.blocks)]))]
    for b in L.blocks:
        parts = L.parts[b["firstPart"]:b["firstPart"] + b["numPars"]]
        ch_rows, ch_nnz = [], []
        for c in range(CH):
            start = b["minRow"]
            end = start
            tot = 0
            for p in parts:
                ck = p["chunks"][c]
                if end < ck["minRow"] + ck["m"]:
                    end = ck["minRow"] + ck["m"]
                tot += ck["e"] - ck["s"]
            ch_rows.append(end - start)
            ch_nnz.append(tot)
        out.append(_word(_u32([b["minRow"], b["minCol"], b["n"], b["numPars"]])))
        out.append(_word(_u32([b["m"], sum(ch_nnz)])))
        out.append(_word(_u16([0] * CH)))          # channel row offsets: always 0
        out.append(_word(_u16(ch_rows)))
        out.append(_u32(ch_nnz))                     # two words
        out.append(b"\0" * (2 * WORD))
    return b"".join(out)


def par_param(L) -> bytes:
    out = [_word(_u32([len(L.parts)]))]
    for p in L.parts:
        base = p["minCol"] // PAR
        ck = p["chunks"]
        out.append(_u32([c["n"] for c in ck]))
        out.append(_u32([c["e"] - c["s"] for c in ck]))
        out.append(_word(_u32([base, -(-p["ncols"] // PAR), p["nrows"], p["rows"].size])))
        out.append(_u16([c["minCol"] // PAR - base for c in ck]))
        out.append(_u16([c["n"] // PAR for c in ck]))
        out.append(b"\0" * WORD)
    return b"".join(out)


def nnz_val(L, data):
    """The 16 channel buffers (gen_nnzStore / update_nnzStore) for values
    data[k] of input position k."""
    data = np.asarray(data, np.float64)
    bufs = []
    row_mod, col_mod = (WORD // 2) * PAR * ACC, (WORD // 2) * PAR
    for c in range(CH):
        body = []
        tot_row = tot_col = tot_nnz = 0
        for b in L.blocks:
            for p in L.parts[b["firstPart"]:b["firstPart"] + b["numPars"]]:
                ck = p["chunks"][c]
                rows = p["rows"][ck["s"]:ck["e"]]
                cols = p["cols"][ck["s"]:ck["e"]]
                src = p["src"][ck["s"]:ck["e"]]
                cnt = rows.size
                tot_row += -(-cnt // row_mod)
                tot_col += -(-cnt // col_mod)
                tot_nnz += cnt // PAR
                ridx = [0] * (WORD // 2)
                cidx = [0] * (WORD // 2)
                r0 = b["minRow"]
                c0 = ck["minCol"] // PAR
                for i in range(0, cnt, PAR):
                    if i % row_mod == 0:
                        for j in range(WORD // 2):
                            if i + j * PAR * ACC < cnt:
                                ridx[j] = int(rows[i + j * PAR * ACC]) - r0
                        body.append(_u16(ridx))
                    if i % col_mod == 0:
                        for j in range(WORD // 2):
                            if i + j * PAR < cnt:
                                cidx[j] = int(cols[i + j * PAR]) // PAR - c0
                        body.append(_u16(cidx))
                    v = [0.0 if s_ < 0 else float(data[s_]) for s_ in src[i:i + PAR]]
                    body.append(np.asarray(v, np.float64).tobytes())
        head = _word(_u32([tot_row + tot_col + tot_nnz, tot_row, tot_col, tot_nnz]))
        bufs.append(head + b"".join(body))
    return bufs


def info(L) -> bytes:
    nnz_pad = sum(p["rows"].size for p in L.parts)
    return _u32([L.m, L.n, L.nnz, L.m, -(-L.n // PAR) * PAR, nnz_pad])


def export(L, data) -> dict:
    """All signature files: {"rbParam", "parParam", "nnzVal_0".."nnzVal_15",
    "info"} -> bytes, as storeMatPar writes them."""
    out = {"rbParam": rb_param(L), "parParam": par_param(L), "info": info(L)}
    for c, buf in enumerate(nnz_val(L, data)):
        out["nnzVal_%d" % c] = buf
    return out


def coo_input(n, row, col, base=0):
    """SparseMatrix::loadCoo: indices minus the base (matrix_params.hpp:51-80)."""
    return np.asarray(row, np.int64) - base, np.asarray(col, np.int64) - base


def cscsym_input(n, rowidx, colptr, data, base=0):
    """SparseMatrix::loadCscSym + SpmPar::getCooDatFromCscSym
    (matrix_params.hpp:82-134, gen_signature.hpp:73-112): entry (i, j) of the
    lower triangle emits (i, j) and, off the diagonal, (j, i), both with its
    value."""
    rowidx = np.asarray(rowidx, np.int64) - base
    colptr = np.asarray(colptr, np.int64) - base
    data = np.asarray(data, np.float64)
    rows, cols, vals = [], [], []
    for j in range(n):
        for k in range(colptr[j], colptr[j + 1]):
            i = int(rowidx[k])
            rows.append(i); cols.append(j); vals.append(data[k])
            if i != j:
                rows.append(j); cols.append(i); vals.append(data[k])
    return np.array(rows, np.int64), np.array(cols, np.int64), np.array(vals, np.float64)
