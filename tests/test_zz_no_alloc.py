"""anacor_absorption_noalloc: the absorption path for callers that cannot
allocate device memory (e.g. code running while another component records a
CUDA graph, or hosts whose device memory is owned by a pool they do not
control).  Its scratch is a fixed file-scope device array, so it must give
the same A_h as the allocating entry point, call after call, and reject
requests that do not fit that array.

This file is collected last on purpose."""
import ctypes as ct

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, synth, tracer

pytestmark = pytest.mark.gpu
RTOL = 1e-6


def _call(L, s, d_label, d_coords, d_out, stream):
    return L.anacor_absorption_noalloc(ct.c_void_p(d_label), np.array(s.label.shape, dtype=np.int64),
                                       ct.c_void_p(d_coords), len(s.coords), np.ascontiguousarray(s.s1),
                                       np.ascontiguousarray(s.omega), s.n_refl, s.xray, s.omega_axis, s.F, s.voxel,
                                       s.mu, 0, 1, ct.c_void_p(d_out), ct.c_void_p(stream))


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    import torch
    build.build()
    L = _lib.load()
    dev = torch.device("cuda")
    stream = torch.cuda.Stream()
    base = synth.small_sample(n_refl=96, seed=3)
    # two different requests in a row: the second must not see the first's leftovers
    cases = [base.subset(refl=slice(0, 96)),
             base.subset(refl=slice(40, 70), coords=base.coords[::2])]
    cases[1].mu = base.mu * 1.7
    d_label = torch.from_numpy(base.label).to(dev)
    for s in cases:
        want = tracer.sample_absorption(s)
        d_coords = torch.from_numpy(np.ascontiguousarray(s.coords)).to(dev)
        d_out = torch.full((s.n_refl,), -1.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = _call(L, s, d_label.data_ptr(), d_coords.data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        assert st == 0, _lib.last_error(L)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.max(np.abs(got - want) / want) <= RTOL


def test_noalloc_rejects_requests_beyond_its_array():
    import torch
    build.build()
    L = _lib.load()
    s = synth.small_sample(n_refl=1)
    n_refl = 60000   # 60k reflection tables alone exceed the 32 MiB array
    s1 = np.tile(s.s1, (n_refl, 1))
    om = np.zeros(n_refl)
    d_label = torch.from_numpy(s.label).cuda()
    d_coords = torch.from_numpy(s.coords).cuda()
    d_out = torch.zeros(n_refl, dtype=torch.float64, device="cuda")
    st = L.anacor_absorption_noalloc(ct.c_void_p(d_label.data_ptr()), np.array(s.label.shape, dtype=np.int64),
                                     ct.c_void_p(d_coords.data_ptr()), len(s.coords), s1, om, n_refl, s.xray,
                                     s.omega_axis, s.F, s.voxel, s.mu, 0, 1, ct.c_void_p(d_out.data_ptr()), None)
    assert st == 3
    assert "scratch" in _lib.last_error(L)[1]
