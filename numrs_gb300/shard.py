"""Sharding of a batch of independent transforms across ranks (one GPU each).

The transforms of a batch are independent -- the crate's
FFTProcessor::fft_batch (src/FFT_1.rs:185-190) runs one rayon task per
transform -- so a batch splits across ranks with no collective on the data
path: every rank transforms its own share in its own persistent launch.

Shares are balanced by the nominal work 5 nn log2 nn of each transform with
the longest-processing-time rule: transforms in decreasing order of work
(ties by index), each one to the rank with the least work so far (ties to the
lower rank).  The partition depends on the sizes and the rank count alone, so
every rank computes the same one without exchanging anything.
"""
import heapq
import math

__all__ = ["transform_work", "partition_by_work"]


def transform_work(nn):
    """Nominal flops of one complex transform of nn points."""
    nn = int(nn)
    return 5.0 * nn * math.log2(nn) if nn > 1 else 0.0


def partition_by_work(sizes, world):
    """Index lists, one per rank (each sorted), covering every transform once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-transform_work(sizes[i]), i))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        w, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (w + transform_work(sizes[i]), r))
    for p in parts:
        p.sort()
    return parts
