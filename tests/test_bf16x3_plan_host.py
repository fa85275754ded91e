"""The tensor-core path's tile plan (ndconv_bf16x3_plan, host only) keeps the
bounds its kernel relies on, over random geometries: the MMA shape
(N = G BN, a multiple of 16 in 16..256), the kernel rows of a group inside
the 128 staged rows for every output row the tile keeps, the K extent
covering the tile's input window, tiles covering the output (a folded
single row: its virtual rows of S outputs), and the
shared memory of the ring, the resident Toeplitz tiles, the epilogue's
blocks and the barriers within the per-CTA limit."""
import ctypes

import numpy as np
import pytest

from ndconv import _abi
from ndconv.api import BorderType, ConvMode, PaddingMode, build_problem, with_dilation

BM, KC = 128, 64
EPILOGUE_AND_BARRIERS = 3 * 128 * 20 * 4 + 256  # + alignment slack


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    return _abi.lib()


def _random_problem(rng):
    rank = int(rng.choice([1, 2, 3], p=[0.2, 0.5, 0.3]))
    shape = tuple(int(rng.integers(1, 300 if rank < 3 else 60)) for _ in range(rank))
    kshape = tuple(int(rng.choice([1, 3, 5, 11, 15, 16, 17, 31, 33, 40, 63, 127])) for _ in range(rank))
    dil = [int(rng.choice([1, 1, 2, 3, 7, 30])) for _ in range(rank)]
    kind = rng.integers(4)
    if kind == 0:
        mode = ConvMode.Full
    elif kind == 1:
        mode = ConvMode.Same
    elif kind == 2:
        mode = ConvMode.Custom([int(rng.integers(0, 40)) for _ in range(rank)],
                               [int(rng.integers(1, 5)) for _ in range(rank)])
    else:
        mode = ConvMode.Explicit([[int(rng.integers(0, 40)), int(rng.integers(0, 40))] for _ in range(rank)],
                                 [int(rng.integers(1, 5)) for _ in range(rank)])
    pm = [PaddingMode.Zeros, PaddingMode.Replicate, PaddingMode.Circular,
          PaddingMode.Custom([BorderType.Zeros] * rank)][int(rng.integers(4))]
    k = np.zeros(kshape, np.float32)
    return build_problem(_abi.F32, shape, with_dilation(k, dil), mode, pm), rank, kshape, dil


def test_tile_plan_bounds(lib):
    rng = np.random.default_rng(2026)
    checked = folded = 0
    for _ in range(3000):
        p, rank, kshape, dil = _random_problem(rng)
        osh = (ctypes.c_int64 * 3)()
        if lib.ndconv_output_shape(ctypes.byref(p), 0, osh) != _abi.OK:
            continue  # kernel larger than the padded input etc.: no plan
        out = (ctypes.c_int64 * 18)()
        st = lib.ndconv_bf16x3_plan(ctypes.byref(p), out)
        if st == _abi.ERR_UNSUPPORTED:
            continue
        assert st == _abi.OK, _abi.last_error()
        G, ng, BN, N, Kpad, nchunk, klast, mvalid, stages, stage_b, ring, smem, bres, nrt, nct, lim, S, R = list(out)
        # canonical axes: the problem's axes in the last `rank` of three
        ks = [1] * (3 - rank) + list(kshape)
        ds = [1] * (3 - rank) + list(dil)
        ss = [1] * (3 - rank) + [int(p.mode_strides[i]) if p.conv_mode >= 3 else 1 for i in range(rank)]
        oo = [1] * (3 - rank) + [int(osh[i]) for i in range(rank)]
        K0, K1, K2 = ks
        assert BN in (16, 32, 64) and N == G * BN and N % 16 == 0 and 16 <= N <= 256
        assert G * ng >= K1 and (ng - 1) * G < K1
        assert mvalid >= 1 and (mvalid - 1) * ss[1] + (G - 1) * ds[1] <= BM - 1
        assert Kpad % 16 == 0 and Kpad >= (BN - 1) * ss[2] + (K2 - 1) * ds[2] + 1
        assert nchunk == (Kpad + KC - 1) // KC and 1 <= klast <= 4 and Kpad == (nchunk - 1) * KC + 16 * klast
        if S:
            # a single row cut into R stretches of S outputs, the last ragged
            assert oo[0] == oo[1] == 1 and K0 == K1 == 1 and S % BN == 0 and R >= 2
            assert (R - 1) * S < oo[2] <= R * S and S * ss[2] >= 4 * (K2 - 1) * ds[2]
            assert nrt * mvalid >= R and nct * BN == S
            folded += 1
        else:
            assert R == 1
            assert nrt * mvalid >= oo[1] and nct * BN >= oo[2]
        assert stages >= 2 and stage_b % 1024 == 0
        bslot = 2 * N * KC * 2
        if bres:
            assert stage_b == 2 * BM * KC * 2 and ring == stages * stage_b + ng * K0 * nchunk * bslot
        else:
            assert stage_b == 2 * BM * KC * 2 + bslot and ring == stages * stage_b
        assert smem >= ring + EPILOGUE_AND_BARRIERS + 1024 and smem <= lim
        checked += 1
    assert checked > 1000 and folded > 100, (checked, folded)


def test_folded_row_reassembles_the_oracle(lib):
    """The single-row fold as the kernel runs it, restated with the oracle:
    with S and R from the library's plan, virtual row r is the padded row's
    positions r S s .. r S s + (S - 1) s + (K - 1) d, each virtual row is
    convolved Valid at the problem's stride (S outputs), and the first
    out outputs of the R S equal the oracle's convolution of the row."""
    from oracle import oracle as O
    rng = np.random.default_rng(77)
    folded = 0
    for _ in range(120):
        n = int(rng.integers(50, 3000))
        K = int(rng.choice([2, 3, 5, 17, 31, 63]))
        d = int(rng.integers(1, 4))
        s = int(rng.integers(1, 4))
        mode = [ConvMode.Full, ConvMode.Same,
                ConvMode.Custom([int(rng.integers(0, 20))], [s]),
                ConvMode.Explicit([[int(rng.integers(0, 30)), int(rng.integers(0, 30))]], [s])][int(rng.integers(4))]
        pm = [PaddingMode.Zeros, PaddingMode.Reflect, PaddingMode.Replicate, PaddingMode.Circular,
              PaddingMode.Const(0.25)][int(rng.integers(5))]
        x = rng.standard_normal(n)
        k = rng.standard_normal(K)
        kw32 = with_dilation(k.astype(np.float32), d)
        p32 = build_problem(_abi.F32, (n,), kw32, mode, pm)
        osh = (ctypes.c_int64 * 3)()
        if lib.ndconv_output_shape(ctypes.byref(p32), 0, osh) != _abi.OK:
            continue
        out = (ctypes.c_int64 * 18)()
        if lib.ndconv_bf16x3_plan(ctypes.byref(p32), out) != _abi.OK:
            continue
        S, R = int(out[16]), int(out[17])
        if not S:
            continue
        p64 = build_problem(_abi.F64, (n,), with_dilation(k, d), mode, pm)
        st, y = O.conv(p64, x, k)
        assert st == 0
        st, xp = O.padding(p64, x)
        assert st == 0
        ss = int(p64.mode_strides[0]) if p64.conv_mode >= 3 else 1
        hop, wv = S * ss, (S - 1) * ss + (K - 1) * d + 1
        rows = np.zeros((R, wv))
        for r in range(R):
            seg = xp[r * hop: r * hop + wv]
            rows[r, :len(seg)] = seg
        # each virtual row: Valid with the problem's stride, zero padding
        pv = build_problem(_abi.F64, (wv,), with_dilation(k, d), ConvMode.Explicit([[0, 0]], [ss]), PaddingMode.Zeros)
        yv = np.concatenate([O.conv(pv, rows[r], k)[1] for r in range(R)])
        assert len(yv) == R * S and (R - 1) * S < len(y) <= R * S
        assert np.allclose(yv[:len(y)], y, rtol=1e-12, atol=1e-12)
        folded += 1
    assert folded > 40, folded
