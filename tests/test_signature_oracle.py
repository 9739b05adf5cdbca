"""CPU checks of the oracle's signature decoder on the committed raw bytes:
the decoded entries of the reference's partitioned matrix equal the stored
order recorded when the fixtures were made, and the transY framing
restatement has the reference's layout."""
import glob
import os
import tempfile

import numpy as np
import pytest

from oracle import sigdecode

RAW = [p for p in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
       if "sig_raw_rbParam" in np.load(p).files]


@pytest.mark.parametrize("path", RAW, ids=lambda p: os.path.basename(p)[:-4])
def test_decoder_on_raw_bytes(path):
    z = np.load(path)
    with tempfile.TemporaryDirectory() as d:
        for k in z.files:
            if k.startswith("sig_raw_"):
                z[k].tofile(os.path.join(d, k[len("sig_raw_"):] + ".dat"))
        so = sigdecode.stored_order(sigdecode.decode(d))
    assert np.array_equal(so["row"], z["sig_row"].astype(so["row"].dtype))
    assert np.array_equal(so["col"], z["sig_col"].astype(so["col"].dtype))
    assert np.array_equal(so["val"], z["sig_val"])


def test_transy_frame_layout():
    y = np.arange(1, 11, dtype=np.float64)
    f = sigdecode.transy_frame(5, 10, y)
    assert len(f) == 64 + 2 * 64
    head = np.frombuffer(f[:64], np.uint32)
    assert head[0] == 5 and head[1] == 10 and not head[2:].any()
    data = np.frombuffer(f[64:], np.float64)
    assert np.array_equal(data[:10], y) and not data[10:].any()
    assert len(sigdecode.transy_frame(0, 0, y)) == 128
