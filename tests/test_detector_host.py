"""Host logic of detector_cut_rows without a GPU: how row arrays become the
SoA columns pt_detector_cut reads (in place for a column-major view,
copied otherwise)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
from petite_gb300.shower import _soa_columns  # noqa: E402

CPU = torch.device("cpu")


def test_column_major_view_is_read_in_place():
    store = torch.arange(4 * 10, dtype=torch.float64).reshape(4, 10)       # a (4, capacity) store
    rows = store[:, :6].T                                                   # (6, 4), strides (1, 10)
    base, stride, first = _soa_columns(rows, 4, CPU)
    assert base.data_ptr() == store.data_ptr() and stride == 10
    assert torch.equal(first, store[0, :6])


def test_row_major_arrays_are_copied_to_soa():
    a = np.arange(24, dtype=np.float64).reshape(6, 4)
    base, stride, first = _soa_columns(a, 4, CPU)
    assert stride == 6 and base.shape == (4, 6) and base.is_contiguous()
    np.testing.assert_array_equal(base.numpy(), a.T)
    np.testing.assert_array_equal(first.numpy(), a[:, 0])


def test_shapes_are_checked():
    with pytest.raises(ValueError):
        _soa_columns(np.zeros((5, 3)), 4, CPU)
    base, stride, _ = _soa_columns(np.zeros((0, 4)), 4, CPU)
    assert stride == 1 and base.shape == (4, 0)
