"""four1 of one transform split across ranks (one GPU each): the four-step
schedule with one all-to-all between the column and the row transforms.

A transform of N = N1 N2 points (powers of two; N1 = 2^floor(log2 N / 2),
N2 = N / N1, both divisible by the rank count P) is read as the N2 x N1 matrix
x[n1 + N1 n2].  With k = k2 + N2 k1, four1's transform (src/FFT_1.rs:5-107,
X_k = sum_n x_n exp(isign 2 pi i n k / N)) factors as

    X[k2 + N2 k1] = sum_n1 w_N1^(n1 k1) w_N^(n1 k2) sum_n2 x[n1 + N1 n2] w_N2^(n2 k2)

with w_M = exp(isign 2 pi i / M).  Layouts of rank r's share (interleaved
complex f64, 2 N / P doubles):

    "columns"  the N1/P columns n1 = r N1/P + c:  share[c, n2] = x[n1 + N1 n2]
    "rows"     the N2/P rows k2 = r N2/P + c:     share[c, k1] = X[k2 + N2 k1]
    "block"    natural order, points [r N/P, (r+1) N/P)

Steps from a "columns" input to a "rows" output:
    1. N1/P transforms of N2 points along the columns    (library: four1_many)
    2. share[c, k2] *= w_N^((r N1/P + c) k2)              (library: twiddle_lines)
    3. all-to-all: columns -> rows of the N2 x N1 spectrum matrix
    4. N2/P transforms of N1 points along the rows        (library: four1_many)
A "block" input adds one all-to-all before step 1, a "block" output one after
step 4.  Between GPUs the exchanges are torch.distributed all_to_all_single
(NCCL); the packing around them is tensor views and copies.

`four1_sharded` runs one rank's share under torch.distributed.
`four1_sharded_local` runs P shares held by one process (one device) with the
exchanges done as copies: the same steps and kernels, for single-GPU tests and
for timing the local work.

fourn (src/Fourn.rs:278 contract, row-major dims n0 x n1 x ...) over slabs:
rank r holds the slabs i0 in [r n0/P, (r+1) n0/P) ("slabs0", a contiguous
block of the array).  It transforms its slabs along axes 1.. (library:
fourn_axes), one all-to-all regroups the array into slabs of axis 1
("slabs1": rank r holds i1 in [r n1/P, (r+1) n1/P), all i0), and the ranks
transform along axis 0.  A "slabs0" output takes one more all-to-all.
`fourn_sharded` / `fourn_sharded_local` as above.
"""
import numpy as np

__all__ = ["split_sizes", "four1_sharded", "four1_sharded_local", "to_layout", "from_layout",
           "fourn_sharded", "fourn_sharded_local", "to_slabs", "from_slabs"]

LAYOUTS = ("columns", "rows", "block")


def split_sizes(N, P):
    """(N1, N2) of the four-step split of N points over P ranks."""
    N = int(N)
    P = int(P)
    if N < 1 or N & (N - 1):
        raise ValueError("N must be a power of two")
    if P < 1 or P & (P - 1):
        raise ValueError("the rank count must be a power of two")
    logn = N.bit_length() - 1
    N1 = 1 << (logn // 2)
    N2 = N // N1
    if N1 % P or N2 % P:
        raise ValueError("N=%d is too small to split over %d ranks" % (N, P))
    return N1, N2


# ---------------------------------------------------------------------------
# The local steps (one share).  `share` is a float64 tensor of 2 N / P values.
# ---------------------------------------------------------------------------
def _transform_lines(share, lines, length, isign, form):
    from . import four1_many
    four1_many(share, length, lines, isign, dist=2 * length, form=form)


def _twiddle(share, lines, length, line0, N, isign):
    from . import twiddle_lines
    twiddle_lines(share, lines, length, line0, N, isign)


def _columns_to_rows_send(share, N1, N2, P):
    """Chunks of a "columns" share for ranks 0..P-1, as one contiguous
    (P, N1/P, N2/P, 2) tensor: chunk s holds the spectrum rows k2 of rank s."""
    return share.view(N1 // P, P, N2 // P, 2).permute(1, 0, 2, 3).contiguous()


def _columns_to_rows_recv(recv, N1, N2, P):
    """A "rows" share from the received (P, N1/P, N2/P, 2) chunks (chunk q
    from rank q: its columns n1 for this rank's rows k2)."""
    return recv.view(P, N1 // P, N2 // P, 2).permute(2, 0, 1, 3).reshape(-1)


def _block_to_columns_send(share, N1, N2, P):
    """A "block" share (rows n2 of the N2 x N1 input) as chunks for the
    column owners: (P, N2/P, N1/P, 2)."""
    return share.view(N2 // P, P, N1 // P, 2).permute(1, 0, 2, 3).contiguous()


def _block_to_columns_recv(recv, N1, N2, P):
    return recv.view(P, N2 // P, N1 // P, 2).permute(2, 0, 1, 3).reshape(-1)


def _rows_to_block_send(share, N1, N2, P):
    """A "rows" share (rows k2, all k1) as chunks for the block owners, whose
    points k = k2 + N2 k1 cover k1 in [s N1/P, (s+1) N1/P): (P, N2/P, N1/P, 2)."""
    return share.view(N2 // P, P, N1 // P, 2).permute(1, 0, 2, 3).contiguous()


def _rows_to_block_recv(recv, N1, N2, P):
    return recv.view(P, N2 // P, N1 // P, 2).permute(2, 0, 1, 3).reshape(-1)


def _check_args(N, isign, in_layout, out_layout):
    if isign not in (1, -1):
        raise ValueError("isign must be +1 or -1")
    if in_layout not in ("columns", "block") or out_layout not in ("rows", "block"):
        raise ValueError("in_layout is 'columns' or 'block', out_layout 'rows' or 'block'")


# ---------------------------------------------------------------------------
# Drivers
# ---------------------------------------------------------------------------
def four1_sharded(share, N, isign, in_layout="columns", out_layout="rows", form="fp64",
                  group=None, transform=None, twiddle=None):
    """This rank's part of a four1 of N points over the ranks of `group`.

    `share` is this rank's 2 N / P doubles in `in_layout` (a CUDA float64
    tensor); returns its 2 N / P doubles in `out_layout` (a new tensor, or
    `share` itself).  `transform(t, lines, length, isign)` and
    `twiddle(t, lines, length, line0, N, isign)` replace the library calls of
    steps 1, 2 and 4 (tests on hosts without a GPU).
    """
    import torch
    import torch.distributed as dist
    _check_args(N, isign, in_layout, out_layout)
    P = dist.get_world_size(group)
    r = dist.get_rank(group)
    N1, N2 = split_sizes(N, P)
    if share.numel() != 2 * N // P:
        raise ValueError("share holds %d doubles, need 2 N / P = %d" % (share.numel(), 2 * N // P))
    tf = transform or (lambda t, lines, length, sg: _transform_lines(t, lines, length, sg, form))
    tw = twiddle or _twiddle

    def exchange(chunks):
        recv = torch.empty_like(chunks)
        dist.all_to_all_single(recv, chunks, group=group)
        return recv

    x = share
    if in_layout == "block":
        x = _block_to_columns_recv(exchange(_block_to_columns_send(x, N1, N2, P)), N1, N2, P)
    x = x.contiguous()
    tf(x, N1 // P, N2, isign)
    tw(x, N1 // P, N2, r * (N1 // P), N, isign)
    x = _columns_to_rows_recv(exchange(_columns_to_rows_send(x, N1, N2, P)), N1, N2, P)
    x = x.contiguous()
    tf(x, N2 // P, N1, isign)
    if out_layout == "block":
        x = _rows_to_block_recv(exchange(_rows_to_block_send(x, N1, N2, P)), N1, N2, P)
    return x


def four1_sharded_local(shares, N, isign, in_layout="columns", out_layout="rows", form="fp64",
                        transform=None, twiddle=None):
    """The same transform for P = len(shares) shares held by this process:
    the steps of four1_sharded, with each all-to-all done as copies."""
    import torch
    _check_args(N, isign, in_layout, out_layout)
    P = len(shares)
    N1, N2 = split_sizes(N, P)
    tf = transform or (lambda t, lines, length, sg: _transform_lines(t, lines, length, sg, form))
    tw = twiddle or _twiddle

    def exchange(chunks):
        # rank s receives chunk s of every rank q, in the order of q
        return [torch.stack([chunks[q][s] for q in range(P)]) for s in range(P)]

    xs = [s.contiguous() for s in shares]
    if in_layout == "block":
        recv = exchange([_block_to_columns_send(x, N1, N2, P) for x in xs])
        xs = [_block_to_columns_recv(t, N1, N2, P).contiguous() for t in recv]
    for r, x in enumerate(xs):
        tf(x, N1 // P, N2, isign)
        tw(x, N1 // P, N2, r * (N1 // P), N, isign)
    recv = exchange([_columns_to_rows_send(x, N1, N2, P) for x in xs])
    xs = [_columns_to_rows_recv(t, N1, N2, P).contiguous() for t in recv]
    for x in xs:
        tf(x, N2 // P, N1, isign)
    if out_layout == "block":
        recv = exchange([_rows_to_block_send(x, N1, N2, P) for x in xs])
        xs = [_rows_to_block_recv(t, N1, N2, P).contiguous() for t in recv]
    return xs


# ---------------------------------------------------------------------------
# Layout helpers (host side, numpy): a natural-order array of N complex values
# (2N doubles) to the P shares of a layout and back.
# ---------------------------------------------------------------------------
def to_layout(x, N, P, layout):
    x = np.asarray(x, dtype=np.float64).reshape(N, 2)
    N1, N2 = split_sizes(N, P)
    if layout == "block":
        return [np.ascontiguousarray(b).reshape(-1) for b in np.split(x, P)]
    if layout == "columns":
        m = x.reshape(N2, N1, 2)  # [n2, n1]
        return [np.ascontiguousarray(m[:, r * (N1 // P):(r + 1) * (N1 // P)].transpose(1, 0, 2)).reshape(-1)
                for r in range(P)]
    if layout == "rows":
        m = x.reshape(N1, N2, 2)  # [k1, k2]
        return [np.ascontiguousarray(m[:, r * (N2 // P):(r + 1) * (N2 // P)].transpose(1, 0, 2)).reshape(-1)
                for r in range(P)]
    raise ValueError("unknown layout %r" % (layout,))


def from_layout(shares, N, layout):
    P = len(shares)
    N1, N2 = split_sizes(N, P)
    parts = [np.asarray(s, dtype=np.float64) for s in shares]
    if layout == "block":
        return np.concatenate(parts)
    if layout == "columns":
        m = np.concatenate([p.reshape(N1 // P, N2, 2) for p in parts])  # [n1, n2]
        return np.ascontiguousarray(m.transpose(1, 0, 2)).reshape(-1)
    if layout == "rows":
        m = np.concatenate([p.reshape(N2 // P, N1, 2) for p in parts])  # [k2, k1]
        return np.ascontiguousarray(m.transpose(1, 0, 2)).reshape(-1)
    raise ValueError("unknown layout %r" % (layout,))


# ---------------------------------------------------------------------------
# fourn over slabs of axis 0
# ---------------------------------------------------------------------------
def _check_slabs(dims, P, isign, out_layout):
    dims = [int(v) for v in dims]
    if len(dims) < 2:
        raise ValueError("fourn over slabs needs two or more dimensions")
    if isign not in (1, -1):
        raise ValueError("isign must be +1 or -1")
    if out_layout not in ("slabs0", "slabs1"):
        raise ValueError("out_layout is 'slabs0' or 'slabs1'")
    if dims[0] % P or dims[1] % P:
        raise ValueError("dims %s do not split over %d ranks along axes 0 and 1" % (dims, P))
    return dims


def _fourn_axes(t, dims, axes, isign, form):
    from . import fourn_axes
    fourn_axes(t, dims, axes, isign, form=form)


def _slabs0_to_slabs1_send(x, dims, P):
    """(n0/P, n1, rest) -> chunks (P, n0/P, n1/P, rest): chunk s holds the
    i1 range of rank s."""
    n0, n1 = dims[0], dims[1]
    rest = x.numel() // (2 * (n0 // P) * n1)
    return x.view(n0 // P, P, n1 // P, rest, 2).permute(1, 0, 2, 3, 4).contiguous()


def _slabs1_to_slabs0_send(x, dims, P):
    """(n0, n1/P, rest) -> chunks (P, n0/P, n1/P, rest): chunk s holds the
    i0 range of rank s."""
    n0, n1 = dims[0], dims[1]
    rest = x.numel() // (2 * n0 * (n1 // P))
    return x.view(P, n0 // P, n1 // P, rest, 2).contiguous()


def _slabs0_from_recv(recv, dims, P):
    """Chunks (P (from rank q: its i1 range), n0/P, n1/P, rest) -> (n0/P, n1, rest)."""
    n0, n1 = dims[0], dims[1]
    return recv.permute(1, 0, 2, 3, 4).reshape(-1)


def fourn_sharded(share, dims, isign, out_layout="slabs1", form="fp64", group=None,
                  transform=None):
    """This rank's part of fourn of a row-major array of dims over the ranks of
    `group`; `share` holds its slabs of axis 0 (a CUDA float64 tensor).
    Returns its part in `out_layout`.  `transform(t, dims, axes, isign)`
    replaces the library's fourn_axes (tests on hosts without a GPU)."""
    import torch
    import torch.distributed as dist
    P = dist.get_world_size(group)
    dims = _check_slabs(dims, P, isign, out_layout)
    tf = transform or (lambda t, d, axes, sg: _fourn_axes(t, d, axes, sg, form))
    local0 = [dims[0] // P] + dims[1:]
    x = share.contiguous()
    tf(x, local0, list(range(1, len(dims))), isign)
    send = _slabs0_to_slabs1_send(x, dims, P)
    recv = torch.empty_like(send)
    dist.all_to_all_single(recv, send, group=group)
    x = recv.reshape(-1)  # chunk q = rank q's i0 range: (n0, n1/P, rest) in order
    local1 = [dims[0], dims[1] // P] + dims[2:]
    tf(x, local1, [0], isign)
    if out_layout == "slabs0":
        send = _slabs1_to_slabs0_send(x, dims, P)
        recv = torch.empty_like(send)
        dist.all_to_all_single(recv, send, group=group)
        x = _slabs0_from_recv(recv, dims, P)
    return x


def fourn_sharded_local(shares, dims, isign, out_layout="slabs1", form="fp64", transform=None):
    """The same for P = len(shares) shares held by this process (exchanges as
    copies)."""
    import torch
    P = len(shares)
    dims = _check_slabs(dims, P, isign, out_layout)
    tf = transform or (lambda t, d, axes, sg: _fourn_axes(t, d, axes, sg, form))
    local0 = [dims[0] // P] + dims[1:]
    xs = [s.contiguous() for s in shares]
    for x in xs:
        tf(x, local0, list(range(1, len(dims))), isign)
    sends = [_slabs0_to_slabs1_send(x, dims, P) for x in xs]
    xs = [torch.stack([sends[q][s] for q in range(P)]).reshape(-1) for s in range(P)]
    local1 = [dims[0], dims[1] // P] + dims[2:]
    for x in xs:
        tf(x, local1, [0], isign)
    if out_layout == "slabs0":
        sends = [_slabs1_to_slabs0_send(x, dims, P) for x in xs]
        xs = [_slabs0_from_recv(torch.stack([sends[q][s] for q in range(P)]), dims, P)
              for s in range(P)]
    return xs


def to_slabs(x, dims, P, layout):
    """A row-major array (2 prod(dims) doubles) as the P shares of a layout."""
    dims = [int(v) for v in dims]
    a = np.asarray(x, dtype=np.float64).reshape(dims + [2])
    ax = 0 if layout == "slabs0" else 1
    return [np.ascontiguousarray(b).reshape(-1) for b in np.split(a, P, axis=ax)]


def from_slabs(shares, dims, layout):
    dims = [int(v) for v in dims]
    P = len(shares)
    ax = 0 if layout == "slabs0" else 1
    shp = list(dims) + [2]
    shp[ax] //= P
    parts = [np.asarray(s, dtype=np.float64).reshape(shp) for s in shares]
    return np.ascontiguousarray(np.concatenate(parts, axis=ax)).reshape(-1)
