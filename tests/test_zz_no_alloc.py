"""plum_cbmc_trials_noalloc (working memory in a fixed array inside the
library, caller-owned device buffers) against plum_cbmc_trials on the same
trial sites, for callers that cannot allocate device memory: a host whose
device memory belongs to its own allocator or budget, or an exchange driver
that cannot take the device-wide synchronisation of cudaMalloc/cudaFree.
Named to be collected last, so that it runs both after the other tests and,
with `pytest tests/test_zz_no_alloc.py`, alone."""
import ctypes as C
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["muvt_neutral", "muvt_charged"]
ERR_INPUT = 1


def _close(a, b):
    # tolerance of the CBMC parity tests: 1e-10 relative, 1e8 = overlap
    if b >= 1e8:
        return a >= 1e8
    return abs(a - b) <= 1e-10 * max(1.0, abs(b))


def _lib():
    import plum_gb300 as pg
    L = pg.lib()
    L.plum_cbmc_trials_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                          C.c_char_p, C.c_int]
    L.plum_cbmc_trials_noalloc.restype = C.c_int
    return L


def _dev(a):
    import torch
    if a is None:
        return None
    return torch.as_tensor(np.ascontiguousarray(a, np.float64)).cuda()


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _noalloc_call(s, T, cl, d, u, did):
    L = _lib()
    err = C.create_string_buffer(256)
    rc = L.plum_cbmc_trials_noalloc(s.h, T, _ptr(d[0]), _ptr(d[1]), cl, _ptr(d[2]), _ptr(d[3]),
                                    did, _ptr(u), err, 256)
    assert rc == 0, (rc, err.value)


def _noalloc_twice(s, b1, b2, chain, ci, did, check_memory=True):
    """Two calls in a row on buffers allocated beforehand; the device's free
    memory (cudaMemGetInfo) is read before and after each call and must not
    change: the entry point allocates nothing. The first call in a process
    also does the entry point's one-time set-up, during which the CUDA
    driver may load the library's code for these kernels (lazy module
    loading); the tests make that call with check_memory=False."""
    import torch
    T = len(b1)
    cl = 0 if chain is None else len(chain)
    d = [_dev(x) for x in (b1, b2, chain, ci)]
    us = [torch.full((T,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for u in us:
        free0 = torch.cuda.mem_get_info()[0]
        _noalloc_call(s, T, cl, d, u, did)
        torch.cuda.synchronize()
        if check_memory:
            assert torch.cuda.mem_get_info()[0] == free0, "device memory changed during the call"
    return [u.cpu().numpy() for u in us]


def _trial_sets(case, seed):
    """Golden grown chains (insertions and deletions) with 32 fresh trial
    sites around each chain end."""
    g = dict(np.load(os.path.join(GOLDEN, case, "cbmc.npz")))
    charged = bool(g["charged"])
    rng = np.random.default_rng(seed)
    off = 0
    for k in range(len(g["u"])):
        cl = int(g["cl"][k])
        chain = g["chain"][off:off + cl]
        ci = g["chain_ci"][off:off + cl]
        off += cl
        base = chain[-1] if cl else g["b1"][k]
        v = rng.normal(size=(32, 3))
        b1 = base + v / np.linalg.norm(v, axis=1)[:, None]
        b2 = rng.uniform(0, 14, size=(32, 3)) if charged else None
        yield (b1, b2, chain if cl else None, ci if (charged and cl) else None,
               int(g["delete_id"][k]))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("form", [0, 1])
def test_noalloc_matches_allocating_entry_point(case, form):
    """The no-alloc entry point always computes with the plain form's FP64
    kernels. On a context of either form, freshly created (its S(k) built
    from scratch in FP64), it must give the plain-form context's
    plum_cbmc_trials energies to 1e-10 relative, on two calls in a row. On a
    precision-form context it is also checked against that context's own
    one-launch FP32 trial kernel at the FP32 tolerance of the CBMC tests
    (1e-4 + 1e-5 |u|)."""
    import plum_gb300 as pg
    d = os.path.join(GOLDEN, case)
    ref = pg.System(d, form=pg.FORM_FP64)
    s = ref if form == 0 else pg.System(d, form=pg.FORM_FP32)
    n = 0
    for k, (b1, b2, chain, ci, did) in enumerate(_trial_sets(case, 11)):
        want = ref.cbmc_trials(b1, b2, chain, ci, did)
        own = s.cbmc_trials(b1, b2, chain, ci, did)
        for got in _noalloc_twice(s, b1, b2, chain, ci, did, check_memory=k > 0):
            for a, b, c in zip(got, want, own):
                assert _close(a, b), (case, form, did, 0 if chain is None else len(chain), a, b)
                if form == 1 and b < 1e8:
                    assert abs(a - c) <= 1e-4 + 1e-5 * abs(a), (case, did, a, c)
        n += 1
    assert n >= 8
    if s is not ref:
        s.close()
    ref.close()


@pytest.mark.gpu
def test_noalloc_rejects_oversize_requests():
    import torch
    import plum_gb300 as pg
    s = pg.System(os.path.join(GOLDEN, "muvt_neutral"))
    L = _lib()
    b = torch.zeros(300 * 3, dtype=torch.float64, device="cuda")
    u = torch.zeros(300, dtype=torch.float64, device="cuda")
    err = C.create_string_buffer(256)
    rc = L.plum_cbmc_trials_noalloc(s.h, 257, _ptr(b), None, 0, None, None, -1, _ptr(u), err, 256)
    assert rc == ERR_INPUT and b"n_trials" in err.value
    rc = L.plum_cbmc_trials_noalloc(s.h, 1, _ptr(b), None, 1025, _ptr(b), None, -1, _ptr(u),
                                    err, 256)
    assert rc == ERR_INPUT and b"chain_len" in err.value
    s.close()
