"""Argument checks of the Python binding that need no GPU: a BlockStream
whose columns disagree in length, or host output columns that cannot hold
the rows the library would write, raise PHJ_ERR_INVALID_ARGUMENT before
any library call."""
import numpy as np
import pytest

import phj_gpu as P


def stream(n=10, types=(P.U32, P.U128)):
    keys = np.arange(n, dtype=np.uint64)
    cols = [np.zeros((n, 2), np.uint64) if t == P.U128 else np.zeros(n, P.TYPE_DTYPE[t]) for t in types]
    return P.BlockStream(list(types), keys, cols)


def test_block_stream_accepts_consistent_columns():
    s = stream()
    assert s.total_rows == 10 and list(s.block_rows) == [10]
    assert P.BlockStream([P.U8], np.arange(25_000, dtype=np.uint64), [np.zeros(25_000, np.uint8)]).block_rows.tolist() == [10_000, 10_000, 5_000]


@pytest.mark.parametrize("bad", ["short_payload", "missing_payload", "block_rows", "keys_2d"])
def test_block_stream_rejects_inconsistent_columns(bad):
    keys = np.arange(10, dtype=np.uint64)
    with pytest.raises(P.PhjError) as e:
        if bad == "short_payload":
            P.BlockStream([P.U32], keys, [np.zeros(9, np.uint32)])
        elif bad == "missing_payload":
            P.BlockStream([P.U32, P.U64], keys, [np.zeros(10, np.uint32)])
        elif bad == "block_rows":
            P.BlockStream([], keys, [], block_rows=np.array([4, 4], np.uint32))
        else:
            P.BlockStream([], keys.reshape(2, 5), [])
    assert e.value.status == P.ERR_INVALID_ARGUMENT


def out_cols(cap, types, dtype_override=None):
    return [np.zeros((cap, 2), np.uint64) if t == P.U128 else np.zeros(cap, dtype_override or P.TYPE_DTYPE[t]) for t in types]


def test_host_output_columns_checked_against_the_schemas():
    b, p = stream(types=(P.U64, P.U128)), stream(types=(P.U16,))
    keys = np.zeros(8, np.uint64)
    lp, rp = P.Context._host_out(b, p, keys, out_cols(8, b.types), out_cols(8, p.types))
    assert lp[0] and lp[1] and rp[0] and not rp[1]
    # longer columns are fine: the capacity is the key column's length
    P.Context._host_out(b, p, keys, out_cols(9, b.types), out_cols(8, p.types))
    bad = [
        (np.zeros(8, np.int64), out_cols(8, b.types), out_cols(8, p.types)),        # key dtype
        (keys, out_cols(7, b.types), out_cols(8, p.types)),                          # a left column too short
        (keys, out_cols(8, b.types)[:1], out_cols(8, p.types)),                      # a left column missing
        (keys, out_cols(8, b.types), out_cols(8, p.types, np.uint32)),               # right column dtype
        (keys, [out_cols(8, b.types)[0], np.zeros(8, np.uint64)], out_cols(8, p.types)),  # u128 column not (n, 2)
        (keys, [np.zeros(16, np.uint64)[::2], out_cols(8, b.types)[1]], out_cols(8, p.types)),  # not contiguous
    ]
    for k, left, right in bad:
        with pytest.raises(P.PhjError) as e:
            P.Context._host_out(b, p, k, left, right)
        assert e.value.status == P.ERR_INVALID_ARGUMENT
