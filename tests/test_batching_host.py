"""The batch order of srf_batch_assemble (simple_rf_gb300/csrc/batch.cu) restated on
the host: a keyed four-round Feistel network on the next power-of-four domain
with cycle walking is a bijection of [0, pool) for every pool size and key, so
an epoch's batches visit distinct rays; different epochs give different orders.
(The device results are compared with the same restatement in
tests/test_gpu_batching.py.)"""
import numpy as np
import pytest

M32 = 0xFFFFFFFF


def mix32(x):
    x &= M32
    x ^= x >> 16
    x = (x * 0x7FEB352D) & M32
    x ^= x >> 15
    x = (x * 0x846CA68B) & M32
    x ^= x >> 16
    return x


def perm_keys(size, seed, epoch):
    bits = 2
    while (1 << bits) < size:
        bits += 1
    half = (bits + 1) // 2
    s0, s1 = seed & M32, (seed >> 32) & M32
    keys = [mix32(s0 ^ mix32(((epoch & M32) * 4 + r + mix32(s1 ^ ((epoch >> 32) & M32))) & M32)) for r in range(4)]
    return keys, half


def permute(pos, size, seed, epoch):
    keys, half = perm_keys(size, seed, epoch)
    mask = (1 << half) - 1
    y = pos
    for _ in range(4096):
        l, r = y >> half, y & mask
        for k in keys:
            l, r = r, l ^ (mix32(r ^ k) & mask)
        y = (l << half) | r
        if y < size:
            return y
    raise AssertionError('walk cap')


def batch_indices(pool, n, seed, counter):
    per_epoch = pool // n
    epoch, b = divmod(counter, per_epoch)
    return [permute(b * n + i, pool, seed, epoch) for i in range(n)]


@pytest.mark.parametrize('size', [4, 5, 7, 64, 100, 1000, 4097, 12345])
def test_order_is_a_bijection(size):
    for seed, epoch in ((0, 0), (7, 3), (2 ** 40 + 5, 11)):
        out = [permute(p, size, seed, epoch) for p in range(size)]
        assert sorted(out) == list(range(size)), (size, seed, epoch)


def test_epochs_visit_distinct_rays_and_reshuffle():
    pool, n = 1000, 128
    per_epoch = pool // n
    e0 = sum((batch_indices(pool, n, 3, b) for b in range(per_epoch)), [])
    e1 = sum((batch_indices(pool, n, 3, b) for b in range(per_epoch, 2 * per_epoch)), [])
    assert len(set(e0)) == len(e0) == per_epoch * n and len(set(e1)) == len(e1)
    assert e0 != e1 and len(set(e0) ^ set(e1)) <= 2 * (pool - per_epoch * n)
