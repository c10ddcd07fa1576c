"""The allocation-free direct sum (tbem_direct_apply_noalloc).

It exists for callers that cannot allocate device memory (a fixed budget
owned by another allocator, real-time loops that cannot afford an
allocation's latency or implicit synchronisation, plugins forbidden to
allocate).  Checked against the allocating entry point tbem_direct_apply,
through the C ABI, on two calls in a row: the second call reuses the shared
static scratch left behind by the first.  Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud(n, seed):
    rng = np.random.default_rng(seed)
    locs = rng.uniform(0, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    return locs, nrm, rng.uniform(0.5, 1.0, n)


@pytest.mark.parametrize("kernel,R", [(0, 1), (3, 3)])
def test_noalloc_direct_matches_allocating_entry_point(kernel, R):
    torch = pytest.importorskip("torch")
    from tbempy import _lib
    L = _lib.lib()
    ol, on, _ = _cloud(1500, 1)
    sl, sn, sw = _cloud(2300, 2)
    params = np.array([1.0, 0.25])
    P = lambda a: C.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else C.c_void_p(a.data_ptr())
    d = {k: torch.tensor(v, device="cuda") for k, v in
         dict(ol=ol, on=on, sl=sl, sn=sn, sw=sw).items()}
    for call in range(2):
        n_rhs = 3 if call == 0 else 1
        x = np.random.default_rng(10 + call).uniform(-1, 1, (n_rhs, R * len(sl)))
        y_ref = np.zeros((n_rhs, R * len(ol)))
        _lib.check(L.tbem_direct_apply(kernel, P(params), P(ol), P(on), len(ol), P(sl), P(sn),
                                       P(sw), len(sl), P(x), P(y_ref), n_rhs, None))
        xd = torch.tensor(x, device="cuda")
        yd = torch.full((n_rhs, R * len(ol)), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(L.tbem_direct_apply_noalloc(kernel, P(params), P(d["ol"]), P(d["on"]), len(ol),
                                               P(d["sl"]), P(d["sn"]), P(d["sw"]), len(sl), P(xd),
                                               P(yd), n_rhs, None))
        torch.cuda.synchronize()
        y = yd.cpu().numpy()
        assert np.linalg.norm(y - y_ref) <= 1e-13 * np.linalg.norm(y_ref)


def test_noalloc_rejects_oversize_and_host_pointers():
    torch = pytest.importorskip("torch")
    from tbempy import _lib
    L = _lib.lib()
    n = 700_000  # R * n_src = 2.1e6 doubles > the 1,966,080 limit
    src = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    w = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    obs = torch.zeros((10, 3), dtype=torch.float64, device="cuda")
    y = torch.zeros(30, dtype=torch.float64, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())
    rc = L.tbem_direct_apply_noalloc(2, None, P(obs), P(obs), 10, P(src), P(src), P(w), n, P(x),
                                     P(y), 1, None)
    assert rc == -1 and b"scratch limit" in L.tbem_last_error()
    host = np.zeros((10, 3))
    rc = L.tbem_direct_apply_noalloc(0, None, C.c_void_p(host.ctypes.data), P(obs), 10, P(obs),
                                     P(obs), P(w), 10, P(x), P(y), 1, None)
    assert rc == -1 and b"device memory" in L.tbem_last_error()
