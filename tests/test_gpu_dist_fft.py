"""The sharded transforms (numrs_gb300.dist) with the library's kernels on
one GPU.  four1: the four-step schedule's local transforms (four1_many), the
twiddle kernel (gbfft_twiddle_lines) and the exchanges, for P = 1, 2 and 4
shares held by one process, and the torch.distributed driver on a one-rank
NCCL group.  fourn over slabs: the axis-subset transform (gbfft_fourn_axes)
and the slab exchange.  Results must match the oracle's four1
(src/FFT_1.rs:5-107) and fourn (src/Fourn.rs:278 contract), or the
single-GPU FP64 transforms, within the FP64 bar."""
import os
import socket

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    pytest.importorskip("torch")
    import numrs_gb300 as nr
    from numrs_gb300 import build
    from numrs_gb300 import dist as D
    build.build()
    return nr, D


@pytest.mark.parametrize("P", [1, 2, 4])
@pytest.mark.parametrize("isign", [1, -1])
@pytest.mark.parametrize("lin,lout", [("columns", "rows"), ("block", "block")])
def test_sharded_local_vs_oracle(env, P, isign, lin, lout):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, D = env
    N = 1 << 20
    x = W.normal(6000 + P, 2 * N)
    ref = x.copy()
    O.four1(ref, N, isign)
    shares = [torch.from_numpy(s.copy()).cuda() for s in D.to_layout(x, N, P, lin)]
    outs = D.four1_sharded_local(shares, N, isign, in_layout=lin, out_layout=lout)
    torch.cuda.synchronize()
    y = D.from_layout([o.cpu().numpy() for o in outs], N, lout)
    e = rel_l2(y, ref)
    assert e <= 1e-12, "sharded four1 2^20 P=%d rel-L2 %.3e" % (P, e)


@pytest.mark.parametrize("P", [2, 4])
def test_sharded_local_2p26_vs_single_gpu(env, P):
    import torch
    from numrs_gb300 import workloads as W
    nr, D = env
    N = 1 << 26
    x = W.normal(6100 + P, 2 * N)
    ref = torch.from_numpy(x).cuda()
    nr.four1(ref, N, 1)
    shares = [torch.from_numpy(s.copy()).cuda() for s in D.to_layout(x, N, P, "block")]
    outs = D.four1_sharded_local(shares, N, 1, in_layout="block", out_layout="block")
    y = torch.cat(outs)
    torch.cuda.synchronize()
    e = float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref))
    assert e <= 1e-12, "sharded four1 2^26 P=%d vs single-GPU rel-L2 %.3e" % (P, e)


@pytest.mark.parametrize("isign", [1, -1])
def test_twiddle_lines_kernel(env, isign):
    import torch
    nr, D = env
    N = 1 << 28
    lines, length, line0 = 8, 1 << 14, (1 << 14) - 5
    rng = np.random.default_rng(6200)
    x = rng.standard_normal(2 * lines * length)
    t = torch.from_numpy(x).cuda()
    nr.twiddle_lines(t, lines, length, line0, N, isign)
    torch.cuda.synchronize()
    c = (x[0::2] + 1j * x[1::2]).reshape(lines, length)
    e = (np.arange(line0, line0 + lines, dtype=np.int64)[:, None] *
         np.arange(length, dtype=np.int64)[None, :]) % N
    want = c * np.exp(isign * 2j * np.pi * (e / N))
    got = t.cpu().numpy()
    gotc = (got[0::2] + 1j * got[1::2]).reshape(lines, length)
    assert np.max(np.abs(gotc - want)) <= 1e-14 * np.max(np.abs(want))


def test_twiddle_lines_rejects(env):
    from numrs_gb300 import _lib as L
    lib = L.load()
    o = L.Opts()
    o.device_ptrs = 0
    x = np.zeros(16)
    # host data is refused; sizes must be powers of two within the tables
    assert lib.gbfft_twiddle_lines(x.ctypes.data, 2, 4, 0, 16, 1, None) == L.INVALID_ARG
    import torch
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    o.device_ptrs = 1
    import ctypes
    o.stream = torch.cuda.current_stream().cuda_stream
    assert lib.gbfft_twiddle_lines(t.data_ptr(), 2, 3, 0, 16, 1, ctypes.byref(o)) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_twiddle_lines(t.data_ptr(), 2, 4, 0, 1 << 30, 1, ctypes.byref(o)) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_twiddle_lines(t.data_ptr(), 2, 4, 0, 16, 0, ctypes.byref(o)) == L.INVALID_ARG


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_sharded_torch_distributed_one_rank(env):
    """four1_sharded's collective path on a one-rank NCCL group."""
    import torch
    import torch.distributed as dist
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, D = env
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(_free_port())})
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        N = 1 << 18
        x = W.normal(6300, 2 * N)
        ref = x.copy()
        O.four1(ref, N, -1)
        out = D.four1_sharded(torch.from_numpy(x).cuda(), N, -1, in_layout="block",
                              out_layout="block")
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref) <= 1e-12
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("axes", [[0], [1], [2], [1, 2], [0, 2], [0, 1, 2]])
@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_fourn_axes(env, axes, form):
    """gbfft_fourn_axes against numpy's FFT along the same axes (fourn's sign:
    isign = -1 is numpy's forward transform)."""
    nr, D = env
    dims = [8, 32, 64]
    n = int(np.prod(dims))
    x = np.random.default_rng(6400).standard_normal(2 * n)
    d = x.copy()
    nr.fourn_axes(d, dims, axes, -1, form=form)
    c = (x[0::2] + 1j * x[1::2]).reshape(dims)
    for ax in axes:
        c = np.fft.fft(c, axis=ax)
    ref = np.stack([c.real, c.imag], axis=-1).reshape(-1)
    e = rel_l2(d, ref)
    assert e <= (1e-12 if form == "fp64" else 1e-6), "fourn_axes %s %s rel-L2 %.3e" % (axes, form, e)


@pytest.mark.parametrize("P", [1, 2, 4])
@pytest.mark.parametrize("lout", ["slabs1", "slabs0"])
def test_fourn_sharded_local_vs_oracle(env, P, lout):
    import torch
    import oracle as O
    nr, D = env
    dims = [16, 32, 64]
    n = int(np.prod(dims))
    x = np.random.default_rng(6500 + P).standard_normal(2 * n)
    ref = x.copy()
    assert O.fourn(ref, dims, 1) == 0
    shares = [torch.from_numpy(s.copy()).cuda() for s in D.to_slabs(x, dims, P, "slabs0")]
    outs = D.fourn_sharded_local(shares, dims, 1, out_layout=lout)
    torch.cuda.synchronize()
    y = D.from_slabs([o.cpu().numpy() for o in outs], dims, lout)
    e = rel_l2(y, ref)
    assert e <= 1e-12, "fourn over %d slabs rel-L2 %.3e" % (P, e)


def test_fourn_sharded_local_c4(env):
    """fourn of 256 x 256 x 512 over 4 slabs against the single-GPU fourn."""
    import torch
    from numrs_gb300 import workloads as W
    nr, D = env
    dims = [256, 256, 512]
    n = int(np.prod(dims))
    x = torch.from_numpy(W.normal(6600, 2 * n)).cuda()
    ref = x.clone()
    nr.fourn(ref, dims, 3, 1)
    shares = list(x.view(4, -1).clone().unbind(0))
    outs = D.fourn_sharded_local(shares, dims, 1, out_layout="slabs0")
    y = torch.cat(outs)
    torch.cuda.synchronize()
    e = float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref))
    assert e <= 1e-12, "fourn C4 over 4 slabs rel-L2 %.3e" % e
