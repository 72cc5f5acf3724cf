"""The sharded transforms of numrs_gb300.dist on two gloo ranks on the CPU:
four1 (four-step schedule, one all-to-all between the column and the row
transforms) and fourn over slabs of axis 0 (one all-to-all between the
transforms of the other axes and axis 0).  The GPU library calls of the local steps are replaced here by numpy
stand-ins (transform = four1's sign convention, twiddle = its definition), so
the test checks the layouts, the exchanges and the twiddle exponents; the
GPU test runs the same steps with the library's kernels.  Reference
transform: four1 of src/FFT_1.rs:5-107 (numpy's FFT with four1's sign)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _four1_np(x, isign):
    """four1's transform of interleaved complex data: X_k = sum x_n e^(isign 2 pi i nk/N)."""
    c = x[0::2] + 1j * x[1::2]
    y = np.fft.ifft(c) * len(c) if isign > 0 else np.fft.fft(c)
    out = np.empty_like(x)
    out[0::2], out[1::2] = y.real, y.imag
    return out


def _np_transform(t, lines, length, isign):
    import torch
    a = t.numpy().reshape(lines, 2 * length)
    for i in range(lines):
        a[i] = _four1_np(a[i].copy(), isign)
    t.copy_(torch.from_numpy(a.reshape(-1)))


def _np_twiddle(t, lines, length, line0, N, isign):
    import torch
    a = t.numpy().reshape(lines, length, 2)
    c = a[..., 0] + 1j * a[..., 1]
    e = (np.arange(line0, line0 + lines)[:, None] * np.arange(length)[None, :]) % N
    c = c * np.exp(isign * 2j * np.pi * e / N)
    out = np.stack([c.real, c.imag], axis=-1)
    t.copy_(torch.from_numpy(np.ascontiguousarray(out).reshape(-1)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, N, isign, lin, lout, x, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from numrs_gb300 import dist as D
    dist.init_process_group("gloo", rank=rank, world_size=world)
    share = torch.from_numpy(D.to_layout(x, N, world, lin)[rank].copy())
    out = D.four1_sharded(share, N, isign, in_layout=lin, out_layout=lout,
                          transform=_np_transform, twiddle=_np_twiddle)
    q.put((rank, out.numpy().copy()))
    dist.destroy_process_group()


@pytest.mark.parametrize("lin,lout", [("columns", "rows"), ("block", "block"), ("block", "rows")])
@pytest.mark.parametrize("isign", [1, -1])
def test_sharded_four1_two_gloo_ranks(lin, lout, isign):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from numrs_gb300 import dist as D
    N, world = 1 << 10, 2
    rng = np.random.default_rng(77)
    x = rng.standard_normal(2 * N)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, N, isign, lin, lout, x, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    y = D.from_layout([got[r] for r in range(world)], N, lout)
    ref = _four1_np(x, isign)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref)) * 10


@pytest.mark.parametrize("P", [1, 2, 4])
def test_sharded_four1_local_emulation_numpy(P):
    """The single-process driver with P shares (exchanges as copies)."""
    pytest.importorskip("torch")
    import torch
    from numrs_gb300 import dist as D
    N = 1 << 12
    x = np.random.default_rng(78).standard_normal(2 * N)
    for lin, lout in (("columns", "rows"), ("block", "block")):
        shares = [torch.from_numpy(s.copy()) for s in D.to_layout(x, N, P, lin)]
        outs = D.four1_sharded_local(shares, N, -1, in_layout=lin, out_layout=lout,
                                     transform=_np_transform, twiddle=_np_twiddle)
        y = D.from_layout([o.numpy() for o in outs], N, lout)
        ref = _four1_np(x, -1)
        assert np.max(np.abs(y - ref)) <= 1e-11 * np.max(np.abs(ref))


def test_layout_round_trip_and_split():
    from numrs_gb300 import dist as D
    N = 1 << 9
    x = np.arange(2 * N, dtype=np.float64)
    for P in (1, 2, 4):
        for lay in D.LAYOUTS:
            assert np.array_equal(D.from_layout(D.to_layout(x, N, P, lay), N, lay), x)
    assert D.split_sizes(1 << 28, 8) == (1 << 14, 1 << 14)
    assert D.split_sizes(1 << 27, 4) == (1 << 13, 1 << 14)
    with pytest.raises(ValueError):
        D.split_sizes(1 << 4, 8)
    with pytest.raises(ValueError):
        D.split_sizes(3 << 4, 2)


def _fourn_np_axes(t, dims, axes, isign):
    """fourn's transform (exp(isign 2 pi i ...), unnormalised) along `axes`."""
    import torch
    a = t.numpy().reshape(list(dims) + [2])
    c = a[..., 0] + 1j * a[..., 1]
    for ax in axes:
        c = np.fft.ifft(c, axis=ax) * dims[ax] if isign > 0 else np.fft.fft(c, axis=ax)
    out = np.stack([c.real, c.imag], axis=-1)
    t.copy_(torch.from_numpy(np.ascontiguousarray(out).reshape(-1)))


def _fourn_rank_main(rank, world, port, dims, isign, lout, x, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from numrs_gb300 import dist as D
    dist.init_process_group("gloo", rank=rank, world_size=world)
    share = torch.from_numpy(D.to_slabs(x, dims, world, "slabs0")[rank].copy())
    out = D.fourn_sharded(share, dims, isign, out_layout=lout, transform=_fourn_np_axes)
    q.put((rank, out.numpy().copy()))
    dist.destroy_process_group()


@pytest.mark.parametrize("dims", [(8, 4, 16), (4, 8), (2, 2, 4, 8)])
@pytest.mark.parametrize("lout", ["slabs1", "slabs0"])
def test_sharded_fourn_two_gloo_ranks(dims, lout):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from numrs_gb300 import dist as D
    world = 2
    n = int(np.prod(dims))
    x = np.random.default_rng(79).standard_normal(2 * n)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_fourn_rank_main, args=(r, world, port, list(dims), -1, lout, x, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    y = D.from_slabs([got[r] for r in range(world)], dims, lout)
    ref = np.zeros_like(x)
    import torch as T
    t = T.from_numpy(x.copy())
    _fourn_np_axes(t, list(dims), list(range(len(dims))), -1)
    ref = t.numpy()
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("P", [1, 2, 4])
def test_sharded_fourn_local_emulation_numpy(P):
    pytest.importorskip("torch")
    import torch
    from numrs_gb300 import dist as D
    dims = [8, 16, 4]
    n = int(np.prod(dims))
    x = np.random.default_rng(80).standard_normal(2 * n)
    t = torch.from_numpy(x.copy())
    _fourn_np_axes(t, dims, [0, 1, 2], 1)
    ref = t.numpy()
    for lout in ("slabs1", "slabs0"):
        shares = [torch.from_numpy(s.copy()) for s in D.to_slabs(x, dims, P, "slabs0")]
        outs = D.fourn_sharded_local(shares, dims, 1, out_layout=lout, transform=_fourn_np_axes)
        y = D.from_slabs([o.numpy() for o in outs], dims, lout)
        assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    with pytest.raises(ValueError):
        D.fourn_sharded_local(shares, [n], 1)  # one dimension: nothing to split
    if P > 1:
        with pytest.raises(ValueError):
            D.fourn_sharded_local(shares, [P // 2, 4 * P, 8], 1)  # axis 0 does not split
