"""Generate the golden vectors in ``reference_vectors.npz`` from numbagg itself.

numbagg compiles its kernels with numba, which is not installed here.  The kernel
bodies are plain Python over numpy arrays, though, and numba compiles them lazily.
So this script puts a names-only ``numba`` stub on ``sys.path``, imports numbagg from
a source checkout, and calls each kernel body directly through the decorator's
``.func`` attribute, e.g. ``numbagg.move_mean.func(a, window, min_count, out)``.

For float64 the Python execution performs the same IEEE operations in the same order
as the numba build without fastmath.  For float32 the moving and exponential kernels
keep float64 locals in numba (``asum = 0.0``) while NumPy 2 would keep float32, so
those kernels are run on the input widened to float64 and the output is rounded to
float32 on store, which is what numba does.  The grouped and matrix kernels
accumulate in the array dtype in both worlds and run unchanged.  numba expands a
constant integer power (``x ** 2``) into multiplications, so every kernel body is
run with that same rewrite applied (see ``_StaticPower``).

Usage (needs a numbagg source tree; the GPU machine does not):

    python tests/golden/make_golden.py [--aggregates-only] /path/to/numbagg-source

It writes ``reference_vectors.npz`` (the scan, fill, grouped and matrix kernels) and
``aggregate_vectors.npz`` (the static aggregations); ``--aggregates-only`` writes the
second alone.  The files are small and committed; tests read them without numbagg.
"""

from __future__ import annotations

import ast
import inspect
import os
import sys
import tempfile
import textwrap
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_vectors.npz")


def _install_numba_stub() -> None:
    class _NT:
        """Stand-in for a numba type: subscriptable, hashable, printable."""

        def __init__(self, name="t", ndim=0):
            self.name, self.ndim = name, ndim

        def __getitem__(self, key):
            nd = len(key) if isinstance(key, tuple) else 1
            return _NT(self.name, nd)

        def __call__(self, *args, **k):
            # `int64(float64)` builds a scalar function signature
            return types.SimpleNamespace(return_type=self, args=args)

        def __repr__(self):
            return self.name

    def _unavailable(*a, **k):
        raise RuntimeError("numba stub: compilation is not available")

    numba = types.ModuleType("numba")
    for nm in ("float32", "float64", "int32", "int64", "int8", "int16", "bool_", "uint8"):
        setattr(numba, nm, _NT(nm))
    numba.guvectorize = _unavailable
    numba.jit = _unavailable
    numba.njit = _unavailable
    numba.from_dtype = lambda dt: _NT(str(dt))
    numba.config = types.SimpleNamespace(THREADING_LAYER="default", THREADING_LAYER_PRIORITY=[])
    core = types.ModuleType("numba.core")
    core_types = types.ModuleType("numba.core.types")
    core_types.Type = _NT
    core.types = core_types
    np_mod = types.ModuleType("numba.np")
    ufunc = types.ModuleType("numba.np.ufunc")
    gufunc = types.ModuleType("numba.np.ufunc.gufunc")
    gufunc.GUFunc = object
    ufunc.gufunc = gufunc
    np_mod.ufunc = ufunc
    numba.core = core
    numba.np = np_mod
    for name, mod in {
        "numba": numba,
        "numba.core": core,
        "numba.core.types": core_types,
        "numba.np": np_mod,
        "numba.np.ufunc": ufunc,
        "numba.np.ufunc.gufunc": gufunc,
    }.items():
        sys.modules[name] = mod


def _import_numbagg(src: str):
    _install_numba_stub()
    sys.path.insert(0, src)
    import numbagg  # noqa: PLC0415

    return numbagg


class _StaticPower(ast.NodeTransformer):
    """Rewrite ``x ** 2`` into ``x * x``.

    numba compiles a float raised to a compile-time integer constant by repeated
    multiplication (its static-power lowering), so ``x ** 2`` is one correctly
    rounded product.  NumPy's scalar ``**`` calls ``pow`` instead, which differs in
    the last bit for about 0.1% of float64 inputs.  Applying the same expansion keeps
    the Python execution identical to the compiled kernels.
    """

    def visit_BinOp(self, node):
        self.generic_visit(node)
        if (
            isinstance(node.op, ast.Pow)
            and isinstance(node.right, ast.Constant)
            and node.right.value == 2
        ):
            return ast.copy_location(
                ast.BinOp(left=node.left, op=ast.Mult(), right=node.left), node
            )
        return node


def _as_compiled(func):
    """The kernel body with numba's static-power expansion applied."""
    src = textwrap.dedent(inspect.getsource(func))
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_StaticPower().visit(tree))
    env = dict(func.__globals__)
    exec(compile(tree, inspect.getsourcefile(func), "exec"), env)
    return env[fdef.name]


def _fixture_array(shape, seed=0):
    """numbagg/test/conftest.py:589-592: rand, values <= 0.1 set to NaN."""
    a = np.random.RandomState(seed).rand(*shape)
    return np.where(a > 0.1, a, np.nan)


def _rows(func_body, arrays, scalars, out_dtype, widen):
    """Run a 1-D kernel body over the rows of 2-D inputs."""
    rows, n = arrays[0].shape
    out = np.empty((rows, n), dtype=np.float64 if widen else out_dtype)
    for r in range(rows):
        row_in = [a[r].astype(np.float64) if widen else a[r] for a in arrays]
        func_body(*row_in, *scalars, out[r])
    return out.astype(out_dtype)


def generate(src: str) -> dict[str, np.ndarray]:
    nb = _import_numbagg(src)
    vec: dict[str, np.ndarray] = {}

    # ---- moving windows ----------------------------------------------------------
    base = _fixture_array((3, 64), seed=0)
    normal = np.random.RandomState(7).randn(2, 64)
    normal[np.random.RandomState(8).rand(2, 64) < 0.1] = np.nan
    b_pair = _fixture_array((3, 64), seed=1)
    move_inputs = {"u": base, "n": normal}
    for dt in ("f64", "f32"):
        dtype = np.float64 if dt == "f64" else np.float32
        for tag, arr in move_inputs.items():
            x = arr.astype(dtype)
            vec[f"move_in_{tag}_{dt}"] = x
            for w in (1, 3, 10, 64):
                for mc in (None, 0, 1, 3):
                    mcv = w if mc is None else mc
                    for fname in ("move_sum", "move_mean", "move_var", "move_std"):
                        f = _as_compiled(getattr(nb, fname).func)
                        vec[f"{fname}|{tag}|{dt}|{w}|{mc}"] = _rows(
                            f, [x], [w, mcv], dtype, widen=(dt == "f32")
                        )
                    if tag == "u":
                        y = b_pair.astype(dtype)
                        vec[f"move_in_b_{dt}"] = y
                        for fname in ("move_cov", "move_corr"):
                            f = _as_compiled(getattr(nb, fname).func)
                            vec[f"{fname}|{tag}|{dt}|{w}|{mc}"] = _rows(
                                f, [x, y], [w, mcv], dtype, widen=(dt == "f32")
                            )

    # known-answer corners from numbagg/test/util.py:41-66 (as 1-row arrays)
    corners = [
        [np.inf, np.nan, 1.0, 2.0],
        [1.0, 2.0, 3.0, 4.0],
        [1e9 + 1, 1e9 + 2, 1e9 + 3, 1e9 + 4],
        [0.0, 0.0, 0.0, 0.0],
        [1.0, np.nan, np.nan, 2.0],
        [np.nan, np.nan, np.nan, np.nan],
    ]
    cor = np.array(corners, dtype=np.float64)
    vec["move_in_corners_f64"] = cor
    for w in (1, 2, 4):
        for fname in ("move_sum", "move_mean", "move_var", "move_std"):
            vec[f"{fname}|corners|f64|{w}|1"] = _rows(
                _as_compiled(getattr(nb, fname).func), [cor], [w, 1], np.float64, widen=False
            )

    # ---- exponentially weighted --------------------------------------------------
    exp_in = _fixture_array((3, 96), seed=2)
    exp_b = _fixture_array((3, 96), seed=3)
    alpha_vec = np.linspace(0.05, 0.9, 96)
    for dt in ("f64", "f32"):
        dtype = np.float64 if dt == "f64" else np.float32
        x = exp_in.astype(dtype)
        y = exp_b.astype(dtype)
        vec[f"exp_in_{dt}"] = x
        vec[f"exp_in_b_{dt}"] = y
        vec[f"exp_alpha_vec_{dt}"] = alpha_vec.astype(dtype)
        for atag, alpha in (("0.5", 0.5), ("0.1", 0.1), ("0.01", 0.01), ("vec", None)):
            al = alpha_vec.astype(dtype) if alpha is None else np.full(96, alpha, dtype=dtype)
            al_run = al.astype(np.float64) if dt == "f32" else al
            for mw in (0.0, 0.5):
                mw_run = float(np.float32(mw)) if dt == "f32" else mw
                for fname in (
                    "move_exp_nancount",
                    "move_exp_nanmean",
                    "move_exp_nansum",
                    "move_exp_nanvar",
                    "move_exp_nanstd",
                ):
                    f = _as_compiled(getattr(nb, fname).func)
                    out = np.empty((3, 96), dtype=np.float64)
                    for r in range(3):
                        xr = x[r].astype(np.float64) if dt == "f32" else x[r]
                        with np.errstate(invalid="ignore", divide="ignore"):
                            f(xr, al_run, mw_run, out[r])
                    vec[f"{fname}|{dt}|{atag}|{mw}"] = out.astype(dtype)
                for fname in ("move_exp_nancov", "move_exp_nancorr"):
                    f = _as_compiled(getattr(nb, fname).func)
                    out = np.empty((3, 96), dtype=np.float64)
                    for r in range(3):
                        xr = x[r].astype(np.float64) if dt == "f32" else x[r]
                        yr = y[r].astype(np.float64) if dt == "f32" else y[r]
                        with np.errstate(invalid="ignore", divide="ignore"):
                            f(xr, yr, al_run, mw_run, out[r])
                    vec[f"{fname}|{dt}|{atag}|{mw}"] = out.astype(dtype)

    # ---- fills -------------------------------------------------------------------
    fill_in = _fixture_array((3, 80), seed=4)
    fill_in[1, 10:30] = np.nan
    fill_in[2, :15] = np.nan
    vec["fill_in_f64"] = fill_in
    vec["fill_in_f32"] = fill_in.astype(np.float32)
    ints = np.random.RandomState(5).randint(-50, 50, size=(2, 40)).astype(np.int32)
    vec["fill_in_i32"] = ints
    for fname in ("ffill", "bfill"):
        f = _as_compiled(getattr(nb, fname).func)
        for lim in (None, 0, 1, 3):
            for dt, arr in (("f64", fill_in), ("f32", fill_in.astype(np.float32)), ("i32", ints)):
                limv = arr.shape[-1] if lim is None else lim
                out = np.empty_like(arr)
                for r in range(arr.shape[0]):
                    f(arr[r], limv, out[r])
                vec[f"{fname}|{dt}|{lim}"] = out

    # ---- grouped -----------------------------------------------------------------
    rs = np.random.RandomState(0)
    labels = rs.choice([-1, 0, 1, 2, 3, 4], size=200)
    vals = rs.rand(2, 200)
    vals = np.where(vals > 0.1, vals, np.nan)
    vals[:, labels == 2] = np.nan  # one group all missing (test_grouped.py:95-99)
    ivals = rs.randint(-100, 100, size=(2, 200)).astype(np.int32)
    bvals = rs.choice([True, False], size=(2, 200))
    vec["group_labels"] = labels.astype(np.int64)
    vec["group_vals_f64"] = vals
    vec["group_vals_f32"] = vals.astype(np.float32)
    vec["group_vals_i32"] = ivals
    vec["group_vals_bool"] = bvals
    no_ints = {"group_nanmean", "group_nanvar", "group_nanstd"}
    no_bool = {"group_nanvar", "group_nanstd"}
    selection_nan = {
        "group_nanargmax",
        "group_nanargmin",
        "group_nanlast",
        "group_nanmin",
        "group_nanmax",
    }
    for fname in nb.GROUPED_FUNCS:
        name = fname.__name__
        body = _as_compiled(fname.func)
        for dt in ("f64", "f32", "i32", "bool"):
            if dt == "bool" and name in no_bool:
                continue
            v = vec[f"group_vals_{dt}"]
            if dt == "bool":
                v = v.astype(np.int32)
            if name in no_ints and v.dtype.kind == "i":
                v = v.astype(np.float64)
            # Integer outputs that the kernel sets to NaN (selection kernels) cannot be
            # written by numpy; numba stores them through fptosi, whose x86-64 result is
            # the type's minimum.  Run those on a float64 buffer and convert the same way.
            nan_int = v.dtype.kind == "i" and name in selection_nan
            for K in (5, 7):
                for ddof in ((0, 1, 5) if name in no_bool else (None,)):
                    out = np.zeros((v.shape[0], K), dtype=np.float64 if nan_int else v.dtype)
                    for r in range(v.shape[0]):
                        with np.errstate(all="ignore"):
                            if ddof is None:
                                body(v[r], labels, out[r])
                            else:
                                body(v[r], labels, ddof, out[r])
                    if nan_int:
                        imin = np.iinfo(v.dtype).min
                        out = np.where(np.isnan(out), imin, out).astype(v.dtype)
                    vec[f"{name}|{dt}|{K}|{ddof}"] = out

    # ---- moving matrices ---------------------------------------------------------
    mat = _fixture_array((24, 4), seed=6)
    vec["matrix_in_f64"] = mat
    vec["matrix_in_f32"] = mat.astype(np.float32)
    for fname in ("move_covmatrix", "move_corrmatrix"):
        body = _as_compiled(getattr(nb, fname).func)
        for dt in ("f64", "f32"):
            a = vec[f"matrix_in_{dt}"]
            for w in (3, 5, 24):
                for mc in (None, 1, 3):
                    mcv = w if mc is None else mc
                    out = np.empty((24, 4, 4), dtype=a.dtype)
                    with np.errstate(all="ignore"):
                        body(a, w, mcv, out)
                    vec[f"{fname}|{dt}|{w}|{mc}"] = out

    # ---- exponentially weighted matrices (numbagg/moving_matrix.py:204-432) -------
    emat = _fixture_array((30, 4), seed=12)
    emat[7, :] = np.nan  # a step with no valid variable
    ealpha = np.linspace(0.05, 0.8, 30)
    for dt in ("f64", "f32"):
        dtype = np.float64 if dt == "f64" else np.float32
        a = emat.astype(dtype)
        vec[f"ematrix_in_{dt}"] = a
        vec[f"ematrix_alpha_vec_{dt}"] = ealpha.astype(dtype)
        for fname in ("move_exp_nancovmatrix", "move_exp_nancorrmatrix"):
            body = _as_compiled(getattr(nb, fname).func)
            for atag in ("0.5", "0.1", "vec"):
                al = ealpha.astype(dtype) if atag == "vec" else np.full(30, float(atag), dtype=dtype)
                for mw in (0.0, 0.5):
                    out = np.empty((30, 4, 4), dtype=dtype)
                    with np.errstate(all="ignore"):
                        body(a, al, dtype(mw), out)
                    vec[f"{fname}|{dt}|{atag}|{mw}"] = out

    # ---- static pairwise-complete matrices (numbagg/funcs.py:338-532) -------------
    smat = _fixture_array((5, 40), seed=13)
    smat[4, :] = np.nan  # a variable with no observation
    smat[3, 2:] = np.nan  # a variable with two observations
    for dt in ("f64", "f32"):
        dtype = np.float64 if dt == "f64" else np.float32
        a = smat.astype(dtype)
        vec[f"smatrix_in_{dt}"] = a
        for fname in ("nancovmatrix", "nancorrmatrix"):
            body = _as_compiled(getattr(nb, fname).func)
            out = np.empty((5, 5), dtype=dtype)
            with np.errstate(all="ignore"):
                body(a, out)
            vec[f"{fname}|{dt}"] = out
    return vec


AGG_OUT = os.path.join(HERE, "aggregate_vectors.npz")


def generate_aggregates(src: str) -> dict[str, np.ndarray]:
    """The static aggregations (numbagg/funcs.py:23-242) run row by row through their
    own kernel bodies: ndaggregate bodies take (row, [ddof,] out[1]), ndreduce bodies
    take a row and return a scalar.  float32 rows run unchanged where numba and NumPy
    type the locals alike (the float32 nansum accumulator, the extremes, the counts) and
    widened to float64 where numba's locals are float64 (nanmean, nanvar, nanstd)."""
    nb = _import_numbagg(src)
    vec: dict[str, np.ndarray] = {}
    f64 = _fixture_array((5, 37), seed=9)
    f64[1, 3] = np.inf
    f64[2, 5] = -np.inf
    f64[3, :] = np.nan  # an all-NaN row (the arg functions use the other rows)
    shifted = 1e6 + np.random.RandomState(10).randn(3, 41)
    shifted[0, ::7] = np.nan
    ints = np.random.RandomState(11).randint(-1000, 1000, size=(4, 29))
    big = np.full((2, 8), 2**30)
    inputs = {
        "f64": f64,
        "f64shift": shifted,
        "f32": f64.astype(np.float32),
        "i32": ints.astype(np.int32),
        "i64": ints.astype(np.int64),
        "i32big": big.astype(np.int32),
    }
    for key, a in inputs.items():
        vec[f"agg_in|{key}"] = a
    widen = {"nanmean", "nanvar", "nanstd"}
    for name in ("allnan", "anynan", "nancount", "nansum", "nanmean", "nanvar", "nanstd"):
        body = _as_compiled(getattr(nb, name).func)
        for key, a in inputs.items():
            if name in widen and a.dtype.kind == "i":
                continue
            for ddof in ((0, 1, 3) if name in ("nanvar", "nanstd") else (None,)):
                res = []
                for r in range(a.shape[0]):
                    row = a[r].astype(np.float64) if (name in widen and a.dtype == np.float32) else a[r]
                    if name in ("allnan", "anynan"):
                        out = np.empty(1, dtype=np.bool_)
                    elif name == "nancount":
                        out = np.empty(1, dtype=np.int64)
                    else:
                        out = np.empty(1, dtype=row.dtype)
                    with np.errstate(all="ignore"):
                        if ddof is None:
                            body(row, out)
                        else:
                            body(row, ddof, out)
                    res.append(out[0])
                dtype = a.dtype if name in ("nansum", "nanmean", "nanvar", "nanstd") else None
                vec[f"agg|{name}|{key}|{ddof}"] = np.array(res, dtype=dtype)
    for name in ("nanmax", "nanmin", "nanargmax", "nanargmin"):
        body = _as_compiled(getattr(nb, name).func)
        for key, a in inputs.items():
            rows = [r for r in range(a.shape[0]) if not (a.dtype.kind == "f" and np.isnan(a[r]).all())]
            if name in ("nanmax", "nanmin"):
                rows = list(range(a.shape[0]))
            with np.errstate(all="ignore"):
                res = [body(a[r]) for r in rows]
            vec[f"agg|{name}|{key}|rows"] = np.array(rows, dtype=np.int64)
            vec[f"agg|{name}|{key}|None"] = np.array(res, dtype=np.int64 if "arg" in name else a.dtype)
    return vec


def _write(vec: dict[str, np.ndarray], path: str) -> None:
    keys = sorted(vec)
    with tempfile.NamedTemporaryFile(dir=HERE, suffix=".npz", delete=False) as fh:
        np.savez_compressed(fh, **{k: vec[k] for k in keys})
        tmp = fh.name
    os.replace(tmp, path)
    print(f"wrote {len(keys)} arrays to {path} ({os.path.getsize(path)} bytes)")


def main() -> None:
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    src = args[0] if args else os.environ.get("NUMBAGG_SRC", "")
    if not src or not os.path.isdir(os.path.join(src, "numbagg")):
        sys.exit("usage: make_golden.py [--aggregates-only] <numbagg source tree>")
    if "--aggregates-only" not in sys.argv:
        _write(generate(src), OUT)
    _write(generate_aggregates(src), AGG_OUT)


if __name__ == "__main__":
    main()
