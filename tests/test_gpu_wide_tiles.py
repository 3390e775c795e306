"""The wide-band LU's tile shapes (gf_solve_opts.wide_tiles, through the C
ABI): rows per CTA of the bulk and of the first trsm, the corner update's tile
edge and rows per CTA of the triangular solves change no entry's arithmetic,
so every shape, and whatever the autotuner picks, solves a plate to the same
bits, in FP64 and in the mixed-precision path."""
import numpy as np
import pytest

from giraffe_gb300 import configs, gpu

pytestmark = pytest.mark.gpu

SHAPES = [(8, 2, 8, 64), (4, 1, 4, 32), (16, 4, 8, 32), (4, 4, 4, 64), (16, 1, 4, 64)]


def _run(ctx, **kw):
    b = gpu.BatchSolver(ctx, [configs.square_plate(12, steps=4), configs.square_plate(5, steps=3, area_update=0)],
                        ctx.opts(**kw))
    b.reset()
    b.run()
    finals, stats = b.results()
    tiles = b.wide_tiles()
    b.close()
    return finals, stats, tiles


@pytest.mark.parametrize("precision", [gpu.GF_PREC_FP64, gpu.GF_PREC_MIXED])
def test_every_tile_shape_gives_the_same_bits(gpu_ctx, precision):
    ref = None
    for shape in SHAPES:
        finals, stats, tiles = _run(gpu_ctx, precision=precision, wide_tiles=shape)
        assert tuple(tiles) == shape
        if ref is None:
            ref = (finals, stats)
            continue
        assert np.array_equal(stats, ref[1]), shape
        for k in range(2):
            assert np.array_equal(finals[k], ref[0][k]), (shape, k)


def test_autotuned_shapes_are_valid_and_change_nothing(gpu_ctx):
    f0, s0, _ = _run(gpu_ctx, wide_tiles=SHAPES[0])
    ft, st, tiles = _run(gpu_ctx)
    assert tiles[0] in (4, 8, 16) and tiles[1] in (1, 2, 4) and tiles[2] in (4, 8) and tiles[3] in (32, 64)
    assert np.array_equal(st, s0)
    for k in range(2):
        assert np.array_equal(ft[k], f0[k]), k
    # the context caches the choice per half-bandwidth
    assert _run(gpu_ctx)[2] == tiles


def test_invalid_tile_shape_is_refused(gpu_ctx):
    with pytest.raises(Exception):
        _run(gpu_ctx, wide_tiles=(3, 2, 8, 64))
