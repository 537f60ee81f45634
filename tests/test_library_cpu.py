"""The C-ABI library: builds, loads, exports every declared symbol, keeps the
host set-up bit-identical to the oracle, and fails loudly without a GPU."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, synth, tracer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "anacor_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"sizeof", "if", "extern", "defined"}
    return sorted({n for n in names if n not in skip and not n.startswith("ANACOR")})


def test_every_declared_symbol_is_exported(lib):
    decl = declared_functions()
    assert "ray_tracing_overall" in decl and "ray_tracing_single" in decl and "ib_test" in decl
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) == set(_lib.EXPORTS)


def test_free_resolves_through_the_library(lib):
    # AnACor's worker frees the result with anacor_lib.free (utils_mp.py:212)
    assert hasattr(lib, "free")


def test_version(lib):
    assert b"sm_103a" in lib.anacor_version()


def test_host_rotation_matches_oracle_bitwise(lib, oracle):
    s = synth.small_sample()
    rx, rs = tracer.rotated_vectors(s.omega_axis, s.omega, s.F, s.xray, s.s1)
    for i in range(s.n_refl):
        xr, sr = oracle.rotate(s, i)
        assert np.array_equal(rx[i], xr) and np.array_equal(rs[i], sr)


def test_ib_test_rejects_a_missing_table(lib):
    s = synth.small_sample(n_refl=1)
    r = lib.ib_test(s.coords, len(s.coords), s.s1[0].copy(), s.xray.copy(), s.voxel, s.mu, None,
                    s.shape, 0, 0, 4)
    assert np.isnan(r)
    assert lib.anacor_last_status() == 3


def _no_gpu():
    import torch
    return not torch.cuda.is_available()


@pytest.mark.skipif(not _no_gpu(), reason="checks the behaviour without a GPU")
def test_no_gpu_means_error_not_fallback(lib):
    s = synth.small_sample(n_refl=3)
    with pytest.raises(_lib.AnacorError):
        tracer.sample_absorption(s)
    from oracle.oracle import row_table
    tab, keep = row_table(s.label)
    res = lib.ray_tracing_overall(0, 3, s.coords, len(s.coords), s.s1, s.omega, s.xray, s.omega_axis, s.F, 3,
                                  s.voxel, s.mu, tab, s.shape, 0, 0, 1, 1)
    assert not res
    assert lib.anacor_last_status() == 4 and lib.anacor_last_error()
