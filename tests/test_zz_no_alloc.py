"""anacor_absorption_noalloc: the absorption path for callers that cannot
allocate device memory (hosts whose device memory is owned by a pool they do
not control, or pipelines that forbid allocation after start-up because
cudaMalloc and cudaFree may synchronise the device).  Its scratch is a fixed
file-scope device array, so it must give the same A_h as the allocating entry
point, call after call, leave the device's free memory unchanged, and reject
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


def test_noalloc_leaves_device_free_memory_unchanged():
    import torch
    build.build()
    L = _lib.load()
    base = synth.small_sample(n_refl=64, seed=5)
    small = base.subset(refl=slice(0, 16), coords=base.coords[::3])
    d_label = torch.from_numpy(base.label).cuda()
    d_big = torch.from_numpy(np.ascontiguousarray(base.coords)).cuda()
    d_small = torch.from_numpy(np.ascontiguousarray(small.coords)).cuda()
    d_out = torch.zeros(base.n_refl, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    # warm-up call: loads the kernels' modules and does the per-device set-up
    assert _call(L, small, d_label.data_ptr(), d_small.data_ptr(), d_out.data_ptr(), stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    # a larger request than the warm-up: more scratch used, no more memory taken
    assert _call(L, base, d_label.data_ptr(), d_big.data_ptr(), d_out.data_ptr(), stream.cuda_stream) == 0, \
        _lib.last_error(L)
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0


def test_noalloc_reports_bad_directions_and_stays_usable():
    import torch
    build.build()
    L = _lib.load()
    s = synth.small_sample(n_refl=8, seed=7)
    d_label = torch.from_numpy(s.label).cuda()
    d_coords = torch.from_numpy(np.ascontiguousarray(s.coords)).cuda()
    d_out = torch.zeros(s.n_refl, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    for bad in (np.nan, np.inf, 0.0):
        t = s.subset(refl=slice(0, 8))
        t.s1 = np.array(s.s1, copy=True)
        t.s1[5] = bad
        st = _call(L, t, d_label.data_ptr(), d_coords.data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        assert st == 7, (bad, _lib.last_error(L))   # ANACOR_ERR_DIRECTION
    # the next good call is unaffected
    want = tracer.sample_absorption(s)
    assert _call(L, s, d_label.data_ptr(), d_coords.data_ptr(), d_out.data_ptr(), stream.cuda_stream) == 0
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    assert np.max(np.abs(got - want) / want) <= RTOL
