"""Device-resident inputs: the structural check that runs before any kernel
indexes through a caller's CSC, for every algorithm and matrix choice, and
the batched workload at a representative scale against the oracle.

The reference performs no such check (assert_col_order only warns,
src/cuda/functions.cu:27-35) and then indexes its slot store out of bounds.
Here a malformed device CSC — offsets that decrease or pass nnz, rows out of
range or out of order, batch instance offsets that do not cover the columns,
a local row outside its instance — returns OPH_ERR_BAD_INPUT and leaves the
context usable.  Every malformed case keeps colptr[m] equal to the length of
the rows buffer, the one fact a caller must get right (no check can see a
buffer's true size)."""
import numpy as np
import pytest

import oracle
from openph_gb300 import complexes as cx
from openph_gb300.api import OPH_ERR_BAD_INPUT, Context, OphError

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def _corrupt(bm, how):
    colptr, rows = bm.colptr.copy(), bm.rows.copy()
    if how == "colptr_decreasing":
        j = int(np.nonzero(np.diff(colptr) > 1)[0][0])  # a column of 2+ rows
        colptr[j + 1] = colptr[j] - 1 if colptr[j] > 0 else colptr[j + 2] + 1
    elif how == "colptr_past_nnz":
        colptr[bm.m // 2] = colptr[-1] + 1000
    elif how == "row_out_of_range":
        rows[-1] = bm.m + 7
    elif how == "rows_not_ascending":
        j = int(np.nonzero(np.diff(colptr) >= 2)[0][-1])
        a = int(colptr[j])
        rows[a], rows[a + 1] = rows[a + 1], rows[a]
    elif how == "negative_row":
        rows[0] = -3
    return colptr, rows


CORRUPTIONS = ["colptr_decreasing", "colptr_past_nnz", "row_out_of_range", "rows_not_ascending", "negative_row"]


@pytest.mark.parametrize("how", CORRUPTIONS)
@pytest.mark.parametrize("algo,dual", [("pms", "never"), ("pms", "auto"), ("pms", "always"), ("twist", "auto"),
                                       ("standard_parallel", "auto"), ("ph_row", "auto")])
def test_malformed_device_csc_rejected(cuda_lib, how, algo, dual):
    torch = pytest.importorskip("torch")
    bm = cx.rips_cube(14, seed=3)
    colptr, rows = _corrupt(bm, how)
    d_colptr, d_rows = _dev(torch, colptr), _dev(torch, rows)
    d_low = torch.empty(bm.m, dtype=torch.int32, device="cuda:0")
    with Context(0) as c:
        c.set_dual(dual)
        torch.cuda.synchronize()
        with pytest.raises(OphError) as e:
            c.reduce_device(bm.m, d_colptr.data_ptr(), d_rows.data_ptr(), d_low.data_ptr(), None, None, algo)
        assert e.value.status == OPH_ERR_BAD_INPUT
        # the context is still usable, and the well-formed matrix reduces exactly
        good_c, good_r = _dev(torch, bm.colptr), _dev(torch, bm.rows)
        torch.cuda.synchronize()
        c.reduce_device(bm.m, good_c.data_ptr(), good_r.data_ptr(), d_low.data_ptr(), None, None, algo)
        np.testing.assert_array_equal(d_low.cpu().numpy(), oracle.twist(bm)[0])


@pytest.mark.parametrize("how", ["offsets_short", "offsets_decreasing", "local_row_past_instance"])
def test_malformed_device_batch_rejected(cuda_lib, how):
    torch = pytest.importorskip("torch")
    mats = [cx.rips_mixed(n, seed=60 + n) for n in (9, 12, 10)]
    col_off = np.cumsum([0] + [bm.m for bm in mats]).astype(np.int64)
    nnz_off = np.cumsum([0] + [bm.nnz for bm in mats]).astype(np.int64)
    colptr = np.concatenate([mats[0].colptr] + [bm.colptr[1:] + nnz_off[b] for b, bm in enumerate(mats) if b > 0])
    rows = np.concatenate([bm.rows for bm in mats])
    total_m, total_nnz = int(col_off[-1]), int(nnz_off[-1])
    if how == "offsets_short":
        col_off[-1] -= 5
    elif how == "offsets_decreasing":
        col_off[1], col_off[2] = col_off[2], col_off[1]
    else:
        # the last row of the first instance points past that instance
        rows[int(nnz_off[1]) - 1] = mats[0].m + 2
    d = [_dev(torch, x) for x in (col_off, colptr, rows)]
    d_low = torch.empty(total_m, dtype=torch.int32, device="cuda:0")
    with Context(0) as c:
        torch.cuda.synchronize()
        with pytest.raises(OphError) as e:
            c.reduce_batch_device(len(mats), d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), total_m, total_nnz,
                                  d_low.data_ptr(), None, "pms")
        assert e.value.status == OPH_ERR_BAD_INPUT


def test_batch_of_256_config_shaped_against_oracle(cuda_lib):
    """256 instances drawn exactly as the 4096-complex batch is (point counts
    uniform in [20, 120], half uniform in the cube and half on a noisy circle,
    full 2-skeleton Rips), ~2.3 * 10^7 columns in one segmented pass through
    the anti-transpose: every instance equals the oracle's twist on it (the
    reference's int32 m * p bound, src/cuda/openph.cu:42, is why the check is
    per instance)."""
    col_off, colptr, rows, npts, _ = cx.rips_mixed_batch(256, seed=9)
    jobs = [(colptr[col_off[b]:col_off[b + 1] + 1] - colptr[col_off[b]],
             rows[colptr[col_off[b]]:colptr[col_off[b + 1]]]) for b in range(256)]
    want = oracle.twist_many(jobs)
    with Context(0) as c:
        low, ess, info = c.reduce_batch_packed(col_off, colptr, rows, "pms")
    assert info["dual"] == 1
    bad = [b for b in range(256) if not (np.array_equal(low[col_off[b]:col_off[b + 1]], want[b][0]) and
                                         np.array_equal(ess[col_off[b]:col_off[b + 1]], want[b][1]))]
    assert bad == [], f"instances differing from the oracle: {bad[:10]}"
    assert npts.min() >= 20 and npts.max() <= 120
