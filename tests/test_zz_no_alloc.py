"""The allocation-free pyramid entry point, cgl_levels_noalloc.

Callers such as hosts that own the GPU memory budget, code recording a CUDA
graph, or frame loops that cannot absorb cudaMalloc's synchronisation use this
entry point; its scratch is a fixed static device array.  Its output must match
the cells the engine's many-body pass builds (read through the engine's own
entry points) bit for bit, on two calls in a row (the second call must not see
the first call's sums).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from graph_gb300 import _abi, generators

from helpers import same_bits

pytestmark = pytest.mark.gpu


def _engine_levels(pos, space):
    from graph_gb300.engine import Engine
    e = Engine(space_size=space, stage_mask=_abi.STAGE_MANYBODY, random_seed=3)
    e.set_point_positions(pos)
    e.render()
    e.start()
    e.step(1)   # the pass bins the positions it starts from: the input positions
    lay = e.layout()
    levels = [e.cells(l)[..., :3].reshape(-1, 3).copy() for l in range(lay.levels)]
    e.close()
    return levels


def _noalloc_levels(lib, pos, space, n_levels, stream):
    import torch
    d_xy = torch.from_numpy(pos).cuda()
    total = sum((4 << l) ** 2 for l in range(n_levels))
    out = torch.full((4 * total,), -1.0, dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    st = lib.cgl_levels_noalloc(d_xy.data_ptr(), pos.size // 2, float(space), out.data_ptr(), out.numel(),
                                stream, err, len(err))
    assert st == _abi.CGL_OK, err.value.decode()
    torch.cuda.synchronize()
    flat = out.cpu().numpy().reshape(-1, 4)
    res, off = [], 0
    for l in range(n_levels):
        g = 4 << l
        res.append(flat[off:off + g * g, :3])
        off += g * g
    return res


def test_noalloc_matches_engine_on_two_calls():
    import torch
    from graph_gb300.engine import load_library
    lib = load_library()
    stream = torch.cuda.current_stream().cuda_stream
    space = 8192.0
    pos_a = generators.uniform_positions(200_000, 0, space, 11)
    pos_b = (4096 + np.random.default_rng(12).normal(0, 300, size=2 * 200_000)).astype(np.float32)
    pos_b[2 * 77] = np.nan                          # an absent point stays out of the grid
    want_a = _engine_levels(pos_a, space)
    want_b = _engine_levels(pos_b, space)
    got_a = _noalloc_levels(lib, pos_a, space, len(want_a), stream)
    got_b = _noalloc_levels(lib, pos_b, space, len(want_b), stream)   # second call in a row
    for want, got in ((want_a, got_a), (want_b, got_b)):
        assert len(want) == len(got) == 8
        for l, (w, g) in enumerate(zip(want, got)):
            assert same_bits(w, g), ("level", l)
    assert got_a[0][:, 2].sum() == 200_000 and got_b[0][:, 2].sum() == 200_000 - 1
    # a third call with fewer levels: its finest level sits elsewhere in the
    # shared array, and only that part is cleared, so the 200k-point sums left
    # there must not leak into it
    pos_c = generators.uniform_positions(3_000, 0, space, 13)
    want_c = _engine_levels(pos_c, space)
    got_c = _noalloc_levels(lib, pos_c, space, len(want_c), stream)
    assert len(want_c) == len(got_c) == 6   # finest grid 128 against the first calls' 512
    for l, (w, g) in enumerate(zip(want_c, got_c)):
        assert same_bits(w, g), ("small call, level", l)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from graph_gb300.engine import load_library
    lib = load_library()
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(16)   # never dereferenced: the sizes are rejected first
    st = lib.cgl_levels_noalloc(dummy, (1 << 24) + 1, 4096.0, dummy, 1 << 30, None, err, len(err))
    assert st == _abi.CGL_INVALID_ARG and b"2^24" in err.value
    st = lib.cgl_levels_noalloc(dummy, 1000, 4096.0, dummy, 16, None, err, len(err))
    assert st == _abi.CGL_INVALID_ARG and b"output holds" in err.value
