"""The dSpmv store side (xJPCG_gbStoreYFrames) against a literal restatement
of the reference's dStoreY loop (dSpmv/hw/include/impl/dStoreY.hpp:36-65),
on frames built by the oracle's transY framing (oracle/sigdecode.py,
transy_frame, after dSpmv/hw/include/impl/transY.hpp:35-65).  Host memory
only: no call here launches device work, so these run without a GPU."""
import numpy as np

import hpc_gb300 as X
from oracle.sigdecode import transy_frame


def dstorey_literal(stream: bytes, num_nodes: int, mem: bytearray):
    """dStoreY as its loops read: per node one 512-bit header word
    {startAddr, rows}, then ceil(rows / 8) 512-bit words, each written as two
    256-bit memory words from memory word startAddr on."""
    pos = 0
    for _ in range(num_nodes):
        head = np.frombuffer(stream, np.uint32, 16, pos)
        pos += 64
        start, rows = int(head[0]), int(head[1])
        mp = start * 32
        for _ in range((rows + 7) // 8):
            dat = stream[pos:pos + 64]
            pos += 64
            for k in range(2):
                mem[mp:mp + 32] = dat[32 * k:32 * k + 32]
                mp += 32
    return pos


def test_store_frames_matches_dstorey_loop():
    rng = np.random.default_rng(7)
    nodes = [(0, 13), (4, 8), (10, 1), (7, 5)]  # (startAddr in 32-byte words, rows); overlaps are legal
    stream = b"".join(transy_frame(s, r, rng.standard_normal(r)) for s, r in nodes)
    y = rng.standard_normal(64)
    mem = bytearray(y.tobytes())
    used_ref = dstorey_literal(stream, len(nodes), mem)
    st, used = X.store_y_frames(stream, len(nodes), y)
    assert st == X.SUCCESS and used == used_ref == len(stream)
    assert y.tobytes() == bytes(mem)  # bit for bit, the zero fill of partial words included


def test_store_frames_round_trip_places_rows():
    rng = np.random.default_rng(8)
    ya, yb = rng.standard_normal(16), rng.standard_normal(24)
    stream = transy_frame(0, 16, ya) + transy_frame(4, 24, yb)  # node 1 at double 16
    y = np.zeros(40)
    st, _ = X.store_y_frames(stream, 2, y)
    assert st == X.SUCCESS
    assert y[:16].tobytes() == ya.tobytes() and y[16:].tobytes() == yb.tobytes()


def test_store_frames_rejects_bad_frames():
    y = np.zeros(16)
    good = transy_frame(0, 8, np.arange(8.0))
    assert X.store_y_frames(good[:-1], 1, y)[0] == X.INVALID_VALUE    # truncated data word
    assert X.store_y_frames(good, 2, y)[0] == X.INVALID_VALUE         # a second header is missing
    assert X.store_y_frames(transy_frame(3, 8, np.arange(8.0)), 1, y)[0] == X.INVALID_VALUE  # writes past y
    assert X.store_y_frames(transy_frame(0, 0, []), 1, y)[0] == X.INVALID_VALUE  # rows = 0
    # frames before a bad one are written, as the FPGA kernel would
    y[:] = 0.0
    st, used = X.store_y_frames(good + transy_frame(9, 8, np.ones(8)), 2, y)
    assert st == X.INVALID_VALUE and used == len(good) and np.array_equal(y[:8], np.arange(8.0))
