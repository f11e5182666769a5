"""Host checks of the index arithmetic the staged kernels rely on (no GPU).

* The Y passes' tensor-map form (kr_fft_y_pipe, kr_ifft_y_pipe in psc_passes.cuh): an array
  of [x][y][kz] complex (H = N/2 + 1) seen as rows of two y, {2H, N N/2} in 8-byte elements.
  A plane tile (TL consecutive kz < N/2 at one x) is the even-row boxes {TL, YB} at kz0 and the
  odd-row boxes {TL + 2, YB} at H - 1 + kz0 (FP32), YB = min(N/2, 256) pairs per box, stacked
  into one staging buffer; thread (t, j) then reads element y = j + r P of line (x, kz0 + t)
  at slot s0 + r sp. Every box start must be a multiple of 16 bytes, every box coordinate in
  range, every shared-memory slot inside the buffer and every slot must hold the element the
  thread expects; plane tiles plus the kz = N/2 column tiles must cover the N H lines with
  the same number of tiles as the direct form.
* The generic engine's planner (plan() in psc_kernels.cu): its tile of TL lines must be a
  power of two (the kernels take a line and an element from the low and high bits of a thread
  index) for every accepted size, with both ping-pong buffers and the Z pass's slots within
  the shared memory of a block.
These restate the formulas of the kernels; they are the checks that were run before the
kernels first ran on a GPU.
"""
import numpy as np
import pytest


def _smooth7(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def _slot(n, t, TL, M, OX=1):
    return TL * M + (n >> 1) * (TL + 2 * OX) + OX + t if n & 1 else (n >> 1) * TL + t


def _y_tile_ok(N, TL):
    H, M, P, OX = N // 2 + 1, N // 2, N // 16, 1
    YB = min(M, 256)
    d0, d1 = 2 * H, N * M                    # the pair view, 8-byte elements (FP32 complex)
    se = (TL + OX) * N                       # staged elements of one array tile
    per = M // TL
    nplane = N * per
    assert nplane + N // TL == -(-N * H // TL)   # the direct form's tile count
    for b in sorted(set(list(range(0, nplane, max(1, nplane // 61))) + [nplane - 1])):
        sm = np.full(se, -1, dtype=np.int64)
        x0, kz0 = b // per, (b % per) * TL
        q0 = x0 * M
        for p0 in range(0, M, YB):
            for odd in (0, 1):
                c0 = (H + kz0 - OX) if odd else kz0
                width = TL + 2 * OX if odd else TL
                base = TL * M + p0 * width if odd else p0 * TL
                assert (c0 * 8) % 16 == 0 and (width * 8) % 16 == 0 and width <= 256 and YB <= 256
                assert (base * 8) % 16 == 0
                for p in range(YB):
                    q = q0 + p0 + p
                    assert 0 <= q < d1
                    for i in range(width):
                        assert 0 <= c0 + i < d0
                        assert base + p * width + i < se
                        sm[base + p * width + i] = q * d0 + c0 + i
        for t in range(TL):
            for j in range(P):
                s0 = _slot(j, t, TL, M)
                sp = (P // 2) * (TL + 2 * OX if j & 1 else TL)
                for r in range(16):
                    n = j + r * P
                    assert s0 + r * sp == _slot(n, t, TL, M)
                    assert sm[s0 + r * sp] == (x0 * N + n) * H + kz0 + t
    return True


@pytest.mark.parametrize("N", [128, 256, 512, 1024])
def test_y_row_pair_tiles(N):
    threads = 512 if N >= 1024 else 256
    TL = threads // (N // 16)
    while TL >= 2:                           # the default tile and the autotuner's narrower ones
        if TL <= N // 2:
            assert _y_tile_ok(N, TL)
        TL //= 2


def test_generic_planner_tiles_are_powers_of_two():
    for N in range(8, 1025, 2):
        pow2 = N & (N - 1) == 0
        if not (pow2 and N < 32) and not (not pow2 and N <= 512 and _smooth7(N)):
            continue                         # the register engine, or a size psc_create refuses
        H, M = N // 2 + 1, N // 2
        for csize in (8, 16):
            tl = 1
            while 2 * tl <= (32768 // csize) // N:
                tl *= 2
            tl = max(tl, 4)
            while tl > 1 and tl // 2 >= N * H:
                tl //= 2
            assert tl & (tl - 1) == 0, (N, csize, tl)
            assert 2 * tl * N * csize <= 227 * 1024
            for nslot in (4, 10, 16):        # Z pass slots: 1, 4 fields with and without GWs
                tlz = 32
                while tlz > 1 and (tlz + 1) * (2 * H + nslot * M) * csize > 100 * 1024:
                    tlz //= 2
                assert (tlz + 1) * (2 * H + nslot * M) * csize <= 227 * 1024, (N, csize, nslot)
