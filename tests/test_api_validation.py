"""Argument checks of the public functions: numbagg's ValueError / TypeError contract
(numbagg/decorators.py:305-341, :374-414, :465-487, :558-674, :778-807), raised
before any device work, so these run on CPU."""

import numpy as np
import pytest

import numbagg_gb300 as nb


@pytest.fixture
def array():
    a = np.random.RandomState(0).rand(3, 500)
    return np.where(a > 0.1, a, np.nan)


def test_move_mean_window(array):
    # numbagg/test/test_moving.py:168-177
    with pytest.raises(TypeError):
        nb.move_mean(array, window=0.5)
    with pytest.raises(ValueError):
        nb.move_mean(array, window=-1)
    with pytest.raises(ValueError):
        nb.move_mean(array, window=array.shape[-1] + 1)
    with pytest.raises(ValueError):
        nb.move_mean(array, window=1, min_count=-1)


@pytest.mark.parametrize("func", [nb.move_sum, nb.move_mean, nb.move_std, nb.move_var])
def test_move_axis_tuple(func, array):
    assert func(array, window=3, axis=()) is array
    with pytest.raises(ValueError, match="only one axis"):
        func(array, window=3, axis=(0, 1))


def test_move_two_arrays_empty_axis(array):
    with pytest.raises(ValueError, match="empty tuple"):
        nb.move_corr(array, array, window=3, axis=())


def test_move_exp_axis(array):
    # numbagg/test/test_moving_exp.py:387-391
    x = np.array([1.0, 2.0, 3.0, 4.0])
    assert nb.move_exp_nansum(x, alpha=0.5, axis=()) is x
    with pytest.raises(ValueError, match="Only one axis"):
        nb.move_exp_nanmean(array, alpha=0.5, axis=(0, 1))
    with pytest.raises(ValueError, match="empty tuple"):
        nb.move_exp_nancorr(array, array, alpha=0.5, axis=())
    with pytest.raises(ValueError, match="alpha has length"):
        nb.move_exp_nanmean(array, alpha=np.full(7, 0.5))


@pytest.mark.parametrize("func", [nb.ffill, nb.bfill])
def test_fill_checks(func, array):
    with pytest.raises(ValueError, match="limit"):
        func(array, limit=-1)
    with pytest.raises(TypeError, match="Unsupported dtype"):
        func(np.array(["a", "b"]), limit=1)
    with pytest.raises(TypeError, match="Unsupported dtype"):
        func(np.array([True, False]))


def test_group_checks():
    values = np.arange(6.0)
    with pytest.raises(TypeError, match="labels must be an integer array"):
        nb.group_nansum(values, np.arange(6.0))
    with pytest.raises(TypeError, match="labels must be an integer array"):
        nb.group_nansum(values, np.arange(6, dtype=np.uint32))
    values2d = np.arange(25.0).reshape(5, 5)
    labels = np.arange(5)
    # numbagg/test/test_grouped.py:270-293
    with pytest.raises(ValueError, match="axis required"):
        nb.group_nansum(values2d, labels)
    with pytest.raises(ValueError, match="must have same shape"):
        nb.group_nansum(values2d, labels[:4], axis=0)
    with pytest.raises(ValueError, match="must have same shape"):
        nb.group_nansum(values2d, labels[:4], axis=(0,))
    # numbagg/test/test_grouped.py:593-603
    for func in (nb.group_nanvar, nb.group_nanstd):
        with pytest.raises(TypeError, match="does not support boolean input"):
            func(np.array([True, False, True]), np.array([0, 0, 1]), num_labels=2)


def test_group_flags_mirror_numbagg():
    assert not nb.group_nanmean.supports_ints
    assert nb.group_nanvar.supports_ddof and not nb.group_nanvar.supports_bool
    assert nb.group_nansum.supports_ints and nb.group_nansum.supports_bool
    assert len(nb.GROUPED_FUNCS) == 15


@pytest.mark.parametrize("func", [nb.move_covmatrix, nb.move_corrmatrix])
def test_move_matrix_checks(func):
    # numbagg/test/test_matrix_functions.py:288-294
    with pytest.raises(ValueError, match="requires at least a 2D array"):
        func(np.array([1, 2, 3, 4, 5], dtype=np.float64), window=3)
    data = np.ones((10, 3))
    with pytest.raises(ValueError, match="window not in valid range"):
        func(data, window=11)
    with pytest.raises(ValueError, match="min_count must be positive"):
        func(data, window=3, min_count=-2)


def test_public_names_match_numbagg_hot_path():
    expected = {
        "move_sum", "move_mean", "move_std", "move_var", "move_cov", "move_corr",
        "move_covmatrix", "move_corrmatrix", "ffill", "bfill",
        "move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar",
        "move_exp_nanstd", "move_exp_nancov", "move_exp_nancorr",
        "group_nanall", "group_nanany", "group_nanargmax", "group_nanargmin", "group_nancount",
        "group_nanfirst", "group_nanlast", "group_nanmax", "group_nanmean", "group_nanmin",
        "group_nanprod", "group_nanstd", "group_nansum", "group_nansum_of_squares", "group_nanvar",
    }
    assert expected <= set(nb.__all__)


@pytest.mark.parametrize(
    "call",
    [
        lambda x: nb.move_mean(x, window=3, precision="fp16"),
        lambda x: nb.move_corr(x, x, window=3, precision="bf16"),
        lambda x: nb.move_exp_nanvar(x, alpha=0.5, precision="double"),
    ],
)
def test_precision_keyword_checked_before_device_work(call):
    # precision= is this package's extension ("f64" default, or "fp32c"); a bad value
    # raises on the host, so no GPU is needed to see it
    with pytest.raises(ValueError, match="precision"):
        call(np.zeros((2, 10)))
