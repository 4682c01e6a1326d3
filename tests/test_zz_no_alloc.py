"""The allocation-free cell sort (jt_cell_sort_noalloc).

Some callers cannot allocate device memory when they call the library (an
application that owns every device allocation through its own pool, or a
time-critical loop that must not call cudaMalloc/cudaFree).  For them the
library offers a variant of the locality sort whose scratch is a fixed array
inside the library.  This file checks, through the C ABI, that two calls in a
row give the same result as the workspace-based jt_cell_sort, and that sizes
beyond the stated maximum are refused.  It is collected last so a failure here
comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from jaxtrace_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 21
MAX_BITS = 6


def _grid(bits):
    g = L.SortGrid()
    g.origin[:] = [-0.25, 0.0, 0.5]
    g.inv_cell[:] = [(1 << bits) / 1.5, (1 << bits) / 1.0, (1 << bits) / 2.0]
    g.bits = bits
    return g


def _morton(pos, g):
    lim = (1 << g.bits) - 1
    c = np.floor((pos - np.array(g.origin[:], np.float32)) * np.array(g.inv_cell[:], np.float32))
    c = np.clip(np.nan_to_num(c), 0, lim).astype(np.int64)
    key = np.zeros(len(pos), np.int64)
    for b in range(g.bits):
        for a in range(3):
            key |= ((c[:, a] >> b) & 1) << (3 * b + a)
    return key


def test_noalloc_sort_matches_workspace_sort_on_two_calls():
    import torch
    assert torch.cuda.is_available()
    lib = L.load()
    st = L.stream_ptr()
    gen = torch.Generator(device="cuda").manual_seed(11)
    for call, (n, bits) in enumerate(((MAX_PARTICLES, MAX_BITS), (777_777, 5))):
        g = _grid(bits)
        lo = torch.tensor(g.origin[:], device="cuda")
        x = (torch.rand((n, 3), device="cuda", generator=gen) * torch.tensor([1.6, 1.1, 2.1], device="cuda") + lo
             - 0.05).contiguous()
        comp = torch.randn((n, 3), device="cuda", generator=gen)
        ids_in = torch.randperm(n, device="cuda", generator=gen).to(torch.int32)
        # the existing entry point, with a caller-allocated workspace
        ws = torch.empty(int(lib.jt_cell_sort_workspace_bytes(n, bits)), dtype=torch.uint8, device="cuda")
        pa, ca, ia = torch.empty_like(x), torch.empty_like(comp), torch.empty_like(ids_in)
        L.check(lib.jt_cell_sort(C.byref(g), n, L.ptr(x), L.ptr(comp), L.ptr(ids_in), L.ptr(pa), L.ptr(ca), L.ptr(ia),
                                 L.ptr(ws), ws.numel(), st))
        # the allocation-free entry point
        pb, cb, ib = torch.empty_like(x), torch.empty_like(comp), torch.empty_like(ids_in)
        L.check(lib.jt_cell_sort_noalloc(C.byref(g), n, L.ptr(x), L.ptr(comp), L.ptr(ids_in), L.ptr(pb), L.ptr(cb),
                                         L.ptr(ib), st))
        torch.cuda.synchronize()
        # same Morton cell sequence slot by slot (tolerance 0: integer keys)
        ka, kb = _morton(pa.cpu().numpy(), g), _morton(pb.cpu().numpy(), g)
        assert np.array_equal(ka, kb), f"call {call}: cell order differs"
        assert np.all(np.diff(kb) >= 0)
        # every particle carried intact with its Kahan terms and id (bit for bit)
        for p_, c_, i_ in ((pa, ca, ia), (pb, cb, ib)):
            src = torch.argsort(i_.long())                    # slot of each original id ...
            order = torch.argsort(ids_in.long())              # ... and its input slot
            assert torch.equal(p_[src], x[order])
            assert torch.equal(c_[src], comp[order])
        assert torch.equal(torch.sort(ia).values, torch.sort(ib).values)


def test_noalloc_sort_rejects_sizes_beyond_its_maximum():
    lib = L.load()
    g = _grid(MAX_BITS)
    with pytest.raises(ValueError, match="at most 2097152 particles"):
        L.check(lib.jt_cell_sort_noalloc(C.byref(g), MAX_PARTICLES + 1, None, None, None, None, None, None, None))
    g7 = _grid(MAX_BITS + 1)
    with pytest.raises(ValueError, match="bits per axis"):
        L.check(lib.jt_cell_sort_noalloc(C.byref(g7), 10, None, None, None, None, None, None, None))
