"""CPU tests of the product's host side: the C ABI library loads and exports
every symbol include/tbem_gpu.h declares, the host octree / task lists are
bit-identical to the reference's (golden fixtures), and argument errors come
back as status codes.  No device compute happens here (host_only plans)."""
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz")))
LISTS = ["p2m", "m2m", "p2p", "m2p", "p2l", "m2l", "l2l", "l2p"]


def header_functions():
    src = open(os.path.join(ROOT, "include", "tbem_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tbem_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from tbempy import _lib
    L = _lib.lib()
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    # and the ctypes table covers exactly the header
    assert sorted(_lib.SIGNATURES) == names


def _header_source():
    src = open(os.path.join(ROOT, "include", "tbem_gpu.h")).read()
    return re.sub(r"/\*.*?\*/", "", src, flags=re.S)


def _ctype_of(decl):
    """The ctypes class the binding must use for one C declaration (a return
    type, or a parameter with its name)."""
    import ctypes as C
    decl = decl.strip()
    if "*" in decl:
        return C.c_char_p if re.fullmatch(r"const\s+char\s*\*", decl) else C.c_void_p
    base = decl.split()[0] if decl.split()[0] != "const" else decl.split()[1]
    return {"int": C.c_int, "long": C.c_long, "double": C.c_double, "void": None}[base]


def test_ctypes_signatures_match_the_header():
    """Every function's return and parameter types in the ctypes table equal
    the header's (int / long / double / pointer), so no argument is truncated
    or widened at the boundary."""
    from tbempy import _lib
    decls = re.findall(r"(int|long|void|const\s+char\s*\*)\s+(tbem_\w+)\s*\(([^)]*)\)\s*;",
                       _header_source())
    assert len(decls) == len(_lib.SIGNATURES)
    for ret, name, params in decls:
        res, args = _lib.SIGNATURES[name]
        params = [p for p in (q.strip() for q in params.split(",")) if p and p != "void"]
        assert res is _ctype_of(ret), name
        assert len(args) == len(params), name
        for a, p in zip(args, params):
            assert a is _ctype_of(p.rsplit(None, 1)[0] + (" *" if "*" in p.rsplit(None, 1)[-1]
                                                          else "")), (name, p)


def test_ctypes_structs_match_the_header():
    """The option and configuration structs: same fields, same order, same
    types as the header's typedefs."""
    from tbempy import _lib
    src = _header_source()
    for cls in (_lib.TbemFmmConfig, _lib.TbemGpuOptions, _lib.TbemIntegrator):
        body = re.search(r"typedef\s+struct\s*\{([^}]*)\}\s*%s\s*;" % cls.__name__, src).group(1)
        fields = [f.strip().rsplit(None, 1) for f in body.split(";") if f.strip()]
        assert [n for _, n in fields] == [n for n, _ in cls._fields_], cls.__name__
        assert [_ctype_of(t) for t, _ in fields] == [t for _, t in cls._fields_], cls.__name__


def test_integration_adapters_compile_against_the_reference(tmp_path):
    """The C++ adapters the integration guide gives a maintainer (an
    OperatorI over the FMM handle, a SparseOperator from the nearfield
    construction) compile against the reference's own headers and
    include/tbem_gpu.h, templates instantiated."""
    import shutil
    import subprocess
    from oracle import oracle
    ref = os.path.join(oracle.REF_ROOT, "cpp")
    gxx = shutil.which("g++")
    if gxx is None or not os.path.isdir(ref):
        pytest.skip("needs g++ and the reference checkout")
    src = tmp_path / "adapter.cpp"
    src.write_text('#include "tbem_operator_adapter.hpp"\n'
                   "template struct tbem::GpuFMMOperator<1>;\n"
                   "template struct tbem::GpuFMMOperator<3>;\n")
    r = subprocess.run([gxx, "-std=c++14", "-fsyntax-only", "-include", "cstddef", "-include",
                        "stdexcept", "-include", "ostream", "-I", ref, "-I",
                        os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_integration_guide_quotes_the_adapter_header():
    """The integration guide's C++ listings are the committed adapter header's
    code, verbatim (so the document cannot drift from what the test above
    compiles)."""
    header = open(os.path.join(ROOT, "include", "tbem_operator_adapter.hpp")).read()
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    assert len(blocks) >= 2
    for b in blocks:
        body = b[b.index("namespace tbem {") + len("namespace tbem {"):b.rindex("}  // namespace tbem")]
        assert body.strip() in header


def kernel_from_name(name, dim=3):
    from tbempy import ThreeD, TwoD
    k = getattr(TwoD if dim == 2 else ThreeD, name)
    return k(1.0, 0.25) if name.startswith("Elastic") else k()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_host_tree_and_lists_match_reference(path):
    from tbempy import ThreeD
    g = dict(np.load(path))
    cfg = ThreeD.FMMConfig(float(g["mac"]), int(g["order"]), int(g["leaf"]), float(g["d"]),
                           bool(g["small"]))
    dim = g["src_locs"].shape[1]
    op = ThreeD.FMMOperator(kernel_from_name(str(g["kernel"]), dim), g["obs_locs"],
                            g["obs_normals"], g["src_locs"], g["src_normals"], g["src_weights"],
                            cfg, host_only=True)
    assert op.n_surface() == int(g["n_surf"])
    for which in (0, 1):
        t = op.tree(which)
        for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
            assert np.array_equal(t[k], g["tree%d_%s" % (which, k)]), k
        assert np.array_equal(np.concatenate(t["indices"]), g["tree%d_indices" % which])
    for kind in LISTS:
        a, b = op.list(kind)
        assert np.array_equal(a, g["list_%s_obs" % kind]), kind
        assert np.array_equal(b, g["list_%s_src" % kind]), kind


def test_host_tree_matches_oracle_on_fault():
    from oracle import oracle
    from tbempy import ThreeD, meshes
    locs, nrm, w, _ = meshes.fault_points(32)
    for small in (False, True):
        cfg = ThreeD.FMMConfig(0.3, 50, 64, 0.05, small)
        op = ThreeD.FMMOperator(ThreeD.ElasticTraction(1.0, 0.25), locs, nrm, locs, nrm, w, cfg,
                                host_only=True)
        orc = oracle.OracleFMM("ElasticTraction", locs, nrm, locs, nrm, w, 0.3, 50, 64, 0.05, small)
        for kind in LISTS:
            for u, v in zip(op.list(kind), orc.list(kind)):
                assert np.array_equal(u, v)


def test_host_tree_and_lists_match_oracle_on_elastic_fault_workload():
    """The elastic fault workload at its stated size (128 x 128 quads, 98,304
    points, 64 points per leaf, MAC 0.3): the product's octree and every task
    list equal the oracle's (itself pinned to the reference's) bit for bit.
    Without small-cell routing the lists do not depend on the kernel or the
    surface order, so the oracle is built with LaplaceSingle at a small order."""
    from oracle import oracle
    from tbempy import ThreeD, meshes
    locs, nrm, w, _ = meshes.fault_points(128, 45.0)
    assert len(locs) == 98304
    cfg = ThreeD.FMMConfig(0.3, 296, 64, 0.05, False)
    op = ThreeD.FMMOperator(ThreeD.ElasticTraction(1.0, 0.25), locs, nrm, locs, nrm, w, cfg,
                            host_only=True)
    orc = oracle.OracleFMM("LaplaceSingle", locs, nrm, locs, nrm, w, 0.3, 6, 64, 0.05, False)
    for which in (0, 1):
        a, b = op.tree(which), orc.tree(which)
        for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
            assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(np.concatenate(a["indices"]), np.concatenate(b["indices"]))
    for kind in LISTS:
        for u, v in zip(op.list(kind), orc.list(kind)):
            assert np.array_equal(u, v), kind
    assert len(op.list("m2l")[0]) > 100000


def test_precision_form_cuts_distinct_trees_from_one_cube():
    """Different observation and source points: the plain form keeps the
    reference's trees (each over its own bounding box), the precision forms
    cut both from the bounding cube of all points, so that every level's
    cells are the same cubes in both trees."""
    from tbempy import ThreeD, meshes
    v, t, obs, on, _, _, _ = meshes.misfit_workload(n=16, n_obs=2000)
    sl, sn, sw = meshes.points_from_mesh(v, t)
    cfg = ThreeD.FMMConfig(0.3, 296, 64, 0.05, False)
    K = ThreeD.ElasticDisplacement(1.0, 0.25)
    for prec in ("mixed", "fp64_compressed"):
        op = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, cfg, precision=prec, host_only=True)
        to, ts = op.tree(1), op.tree(0)
        root = to["hw"][0]
        assert root[0] == root[1] == root[2] and np.array_equal(ts["hw"][0], root)
        assert np.array_equal(to["center"][0], ts["center"][0])
        for tr in (to, ts):
            assert np.array_equal(tr["hw"], root[None, :] * 2.0 ** -tr["level"][:, None])
    plain = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, cfg, host_only=True)
    assert not np.array_equal(plain.tree(1)["hw"][0], plain.tree(0)["hw"][0])


def test_degenerate_inputs_build():
    """Coincident and nearly coincident points (unit_tests/test_octree.cpp:113-125)."""
    from tbempy import ThreeD
    cfg = ThreeD.FMMConfig(0.3, 6, 1, 0.05, False)
    for pts in (np.array([[1.0, 2.0, 0.0], [1.0, 2.0, 0.0]]),
                np.array([[1.0, 2.0, 0.0], [1.0, 2.0 - 1e-20, 0.0], [0.0, 0.0, 0.0]])):
        op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), pts, pts, pts, pts, np.ones(len(pts)),
                                cfg, host_only=True)
        t = op.tree(0)
        assert t["n_idx"][0] == len(pts)


def test_empty_meshes_build():
    """Empty meshes must not error (acceptance_tests/test_empty_operator.py:10-17)."""
    from tbempy import ThreeD
    e = np.zeros((0, 3))
    cfg = ThreeD.FMMConfig(0.3, 20, 10, 0.05, False)
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), e, e, e, e, np.zeros(0), cfg, host_only=True)
    assert op.n_rows() == 0 and op.n_cols() == 0


def test_argument_errors_are_status_codes():
    from tbempy import ThreeD
    from tbempy._lib import TbemError
    p = np.random.default_rng(0).uniform(0, 1, (10, 3))
    with pytest.raises(TbemError) as e:
        ThreeD.FMMOperator(ThreeD.LaplaceSingle(), p, p, p, p, np.ones(10),
                           ThreeD.FMMConfig(0.3, 20, 0, 0.05, False), host_only=True)
    assert e.value.code == -1 and "min_pts" in str(e.value)

    class Bad(ThreeD.Kernel):
        kernel_id = 42
    with pytest.raises(TbemError):
        ThreeD.FMMOperator(Bad(), p, p, p, p, np.ones(10),
                           ThreeD.FMMConfig(0.3, 20, 5, 0.05, False), host_only=True)
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), p, p, p, p, np.ones(10),
                            ThreeD.FMMConfig(0.3, 20, 5, 0.05, False), host_only=True)
    with pytest.raises(TbemError) as e:
        op.apply(np.ones(10))
    assert e.value.code == -4
    # a clone rebuilds the same tree and lists
    c = op.clone()
    assert c.n_rows() == op.n_rows() and c.n_cols() == op.n_cols()
    for kind in range(8):
        assert all(np.array_equal(a, b) for a, b in zip(op.list(kind), c.list(kind)))
    for which in (0, 1):
        assert np.array_equal(op.tree(which)["center"], c.tree(which)["center"])

    # the direct sum refuses null arrays before touching the device
    import ctypes as C
    from tbempy import _lib
    L = _lib.lib()
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    y = np.zeros(10)
    assert L.tbem_direct_apply(0, None, P(p), P(p), 10, P(p), P(p), None, 10, P(y), P(y), 1,
                               None) == -1
    assert "null" in L.tbem_last_error().decode()
    # the gradient entry points check their arguments before any device use
    assert L.tbem_fmm_observation_gradients(None, P(y), P(y), None, None, None) == -1
    assert L.tbem_fmm_source_gradients(None, P(y), P(y), None, None, None, None) == -1
    # the setup cache is host memory: emptying it needs no device
    ThreeD.clear_setup_cache()


def test_2d_operators_build_quadtrees_and_refuse_the_precision_form():
    """2D kernels: quadtrees over x and y with the reference's lists (checked
    against the oracle, itself pinned to the reference), n_rows = R n_obs,
    empty and coincident inputs, and the precision form refused with a
    status (it rests on the 3D kernels' homogeneity)."""
    from oracle import oracle
    from tbempy import ThreeD, TwoD
    from tbempy._lib import TbemError
    rng = np.random.default_rng(9)
    src, obs = rng.uniform(-1, 1, (900, 2)), rng.uniform(-1, 1, (500, 2)) * 0.7
    ns = rng.normal(size=(900, 2))
    no = rng.normal(size=(500, 2))
    w = rng.uniform(0.5, 1, 900)
    for small in (False, True):
        cfg = ThreeD.FMMConfig(0.3, 16, 12, 0.05, small)
        for K in (TwoD.LaplaceHypersingular(), TwoD.ElasticTraction(1.0, 0.25)):
            op = TwoD.FMMOperator(K, obs, no, src, ns, w, cfg, host_only=True)
            assert op.n_rows() == K.tensor_dim * 500 and op.n_cols() == K.tensor_dim * 900
            assert op.n_surface() == 16
            orc = oracle.OracleFMM(K.kernel_id, obs, no, src, ns, w, 0.3, 16, 12, 0.05, small)
            for which in (0, 1):
                t, u = op.tree(which), orc.tree(which)
                assert t["n_children"].max() <= 4
                for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
                    assert np.array_equal(t[k], u[k]), k
            for kind in LISTS:
                for a, b in zip(op.list(kind), orc.list(kind)):
                    assert np.array_equal(a, b), kind
    e = np.zeros((0, 2))
    op = TwoD.FMMOperator(TwoD.LaplaceSingle(), e, e, e, e, np.zeros(0),
                          ThreeD.FMMConfig(0.3, 8, 10, 0.05, False), host_only=True)
    assert op.n_rows() == 0
    same = np.array([[1.0, 2.0], [1.0, 2.0], [0.0, 0.0]])
    op = TwoD.FMMOperator(TwoD.LaplaceSingle(), same, same, same, same, np.ones(3),
                          ThreeD.FMMConfig(0.3, 8, 1, 0.05, False), host_only=True)
    assert op.tree(0)["n_idx"][0] == 3
    with pytest.raises(TbemError) as err:
        TwoD.FMMOperator(TwoD.LaplaceSingle(), src, ns, src, ns, w,
                         ThreeD.FMMConfig(0.3, 16, 12, 0.05, False), precision="mixed",
                         host_only=True)
    assert err.value.code == -1 and "2D" in str(err.value)


def test_csr_create_validates():
    from tbempy import ThreeD
    from tbempy._lib import TbemError
    with pytest.raises(TbemError):
        ThreeD.SparseOperator(2, 2, [1.0], [5], [0, 1, 1])   # column out of range
    with pytest.raises(TbemError):
        ThreeD.SparseOperator(2, 2, [1.0, 2.0], [0, 1], [0, 2, 1])  # decreasing row_ptrs
    # the column check runs in blocks of 2^20 entries on all host cores: a bad
    # column in the last of several blocks (or a negative one in the first)
    nnz = 3 * (1 << 20) + 5
    cols = np.zeros(nnz, dtype=np.int64)
    for k, bad in ((nnz - 1, 7), (3, -1)):
        c = cols.copy()
        c[k] = bad
        with pytest.raises(TbemError) as e:
            ThreeD.SparseOperator(1, 7, np.ones(nnz), c, [0, nnz])
        assert "column" in str(e.value)


def test_graph_arguments_rejected_before_device_use():
    """tbem_fmm_graph_create validates its arguments before any device call:
    no operators, a null operator, a host_only operator or n_rhs <= 0 come
    back as status codes with a message."""
    import ctypes as C
    from tbempy import ThreeD, _lib
    L = _lib.lib()
    h = C.c_void_p()
    assert L.tbem_fmm_graph_create(None, 0, None, None, 1, 0, C.byref(h)) == -1
    assert h.value is None and b"no operators" in L.tbem_last_error()
    rng = np.random.default_rng(0)
    locs = rng.uniform(0, 1, (100, 3))
    nrm = np.tile([0.0, 0.0, 1.0], (100, 1))
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), locs, nrm, locs, nrm, np.ones(100),
                            ThreeD.FMMConfig(0.3, 20, 20, 0.05, False), host_only=True)
    ops = (C.c_void_p * 1)(op._h.value)
    ptrs = (C.c_void_p * 1)(0)
    assert L.tbem_fmm_graph_create(ops, 1, ptrs, ptrs, 0, 0, C.byref(h)) == -1  # n_rhs
    nulls = (C.c_void_p * 1)(None)
    assert L.tbem_fmm_graph_create(nulls, 1, ptrs, ptrs, 1, 0, C.byref(h)) == -1
    assert L.tbem_fmm_graph_create(ops, 1, ptrs, ptrs, 1, 0, C.byref(h)) == -4  # host_only
    assert b"host_only" in L.tbem_last_error()
    assert L.tbem_fmm_graph_launch(None, None) == -1


def test_header_and_library_from_plain_c(tmp_path):
    """include/tbem_gpu.h is a C header: a C99 program compiles against it,
    links with the library and builds a host-only operator through the ABI
    (trees and lists only, no device use)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from tbempy import _lib
    lib_path = _lib.lib()._name
    src = tmp_path / "abi.c"
    src.write_text(r"""
#include <stdio.h>
#include "tbem_gpu.h"
int main(void) {
    double locs[3 * 64], nrm[3 * 64], w[64];
    for (int i = 0; i < 64; i++) {
        locs[3 * i] = (i % 4) * 0.25; locs[3 * i + 1] = ((i / 4) % 4) * 0.25;
        locs[3 * i + 2] = (i / 16) * 0.25;
        nrm[3 * i] = 0; nrm[3 * i + 1] = 0; nrm[3 * i + 2] = 1; w[i] = 1.0;
    }
    TbemFmmConfig cfg = {0.3, 20, 8, 0.05, 0};
    TbemGpuOptions opt;
    tbem_default_options(&opt);
    opt.host_only = 1;
    TbemFmm* h = NULL;
    int rc = tbem_fmm_create(TBEM_LAPLACE_SINGLE, NULL, locs, nrm, 64, locs, nrm, w, 64, &cfg, &opt, &h);
    if (rc != TBEM_OK) { printf("create failed: %s\n", tbem_last_error()); return 1; }
    long cells = tbem_fmm_tree_cells(h, 0, NULL, NULL, NULL, NULL, NULL, NULL);
    double x[64], y[64];
    int rc2 = tbem_fmm_apply(h, x, y, 1, NULL);   /* host_only: refused with a status */
    printf("%ld %ld %ld %d\n", tbem_fmm_n_rows(h), tbem_fmm_n_cols(h), cells, rc2 == TBEM_ERR_STATE);
    tbem_fmm_destroy(h);
    return 0;
}
""")
    exe = tmp_path / "abi"
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(lib_path)
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", inc, str(src), "-o", str(exe),
                    "-L", libdir, "-ltbem_gpu", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out[0] == "64" and out[1] == "64" and int(out[2]) > 1 and out[3] == "1"
