"""Position hand-off in the renderer's texture layout (Points/position-utils.ts:9-27)."""
import numpy as np
import pytest

from helpers import make_pair, scenario

pytestmark = pytest.mark.gpu


def _expected(xy, t):
    n = xy.size // 2
    tex = np.zeros((t * t, 4), dtype=np.float32)
    tex[:n, 0] = xy[0::2]
    tex[:n, 1] = xy[1::2]
    tex[:n, 2] = np.arange(n, dtype=np.float32)
    return tex


def _same(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32)) or \
        (np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]))


def test_texture_layout_host_pinned_device():
    torch = pytest.importorskip("torch")
    pos, links, fields = scenario("ba_small")
    pos = pos.copy()
    pos[2 * 5: 2 * 8] = np.nan                 # absent points read NaN, keep their index
    n = pos.size // 2
    eng, orc = make_pair(pos, links, fields)
    eng.step(3)
    orc.step(3)
    t = eng.layout().points_texture_size
    assert t * t >= n and (t - 1) * (t - 1) < n
    want = _expected(orc.get_point_positions(), t)
    got = eng.get_position_texture()                                 # pageable host memory
    assert _same(got, want)
    pinned = torch.empty(4 * t * t, dtype=torch.float32, pin_memory=True)
    eng.get_position_texture_into(pinned.data_ptr(), pinned.numel())  # written by the kernel itself
    assert _same(pinned.numpy().reshape(-1, 4), want)
    dev = torch.full((4 * t * t,), 7.0, dtype=torch.float32, device="cuda")
    eng.enqueue_position_texture(dev.data_ptr(), dev.numel())
    eng.synchronize()
    assert _same(dev.cpu().numpy().reshape(-1, 4), want)


def test_queued_snapshots_between_ticks():
    torch = pytest.importorskip("torch")
    pos, links, fields = scenario("collision")
    eng, orc = make_pair(pos, links, fields)
    t = eng.layout().points_texture_size
    snaps = [torch.empty(4 * t * t, dtype=torch.float32, pin_memory=True) for _ in range(3)]
    for s in snaps:           # no stall between the ticks: each snapshot is queued after its tick
        eng.step(1)
        eng.enqueue_position_texture(s.data_ptr(), s.numel())
    eng.synchronize()
    for s in snaps:
        orc.step(1)
        assert _same(s.numpy().reshape(-1, 4), _expected(orc.get_point_positions(), t))


def test_texture_rejects_small_buffers():
    from graph_gb300._calls import StatusError
    pos, links, fields = scenario("center")
    eng, orc = make_pair(pos, links, fields)
    out = np.empty(8, dtype=np.float32)
    with pytest.raises(StatusError):
        eng.get_position_texture_into(out.ctypes.data, out.size)
    with pytest.raises(StatusError):          # pageable memory cannot be written asynchronously
        t = eng.layout().points_texture_size
        big = np.empty(4 * t * t, dtype=np.float32)
        eng.enqueue_position_texture(big.ctypes.data, big.size)


def test_positions_into_pinned_memory():
    # read-back into pinned host memory (the e2e path), at 16- and 8-byte alignment
    torch = pytest.importorskip("torch")
    pos, links, fields = scenario("center")
    pos = np.concatenate([pos, np.float32([1.5, 2.5])])       # an odd number of points
    eng, orc = make_pair(pos, links, fields)
    eng.step(2)
    want = eng.get_point_positions()
    n = want.size
    pinned = torch.empty(n, dtype=torch.float32, pin_memory=True)
    eng.get_point_positions_into(pinned.numpy())
    assert _same(pinned.numpy(), want)
    off = torch.empty(n + 2, dtype=torch.float32, pin_memory=True)   # 8- but not 16-byte aligned view
    eng.get_point_positions_into(off.numpy()[2:])
    assert _same(off.numpy()[2:], want)
    orc.step(2)
    assert _same(want, orc.get_point_positions())


def test_queued_point_positions_beside_the_ticks():
    # cgl_enqueue_point_positions: each call's copy lands by the next call (two
    # buffers alternate), the last by synchronize; every tick's positions equal
    # the synchronous read-back's and the oracle's
    torch = pytest.importorskip("torch")
    from graph_gb300._calls import StatusError
    pos, links, fields = scenario("collision")
    eng, orc = make_pair(pos, links, fields)
    n = eng.layout().points_number
    bufs = [torch.empty(2 * n, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    got = []
    for k in range(6):
        eng.step(1)
        eng.enqueue_point_positions_into(bufs[k % 2].numpy())
        if k:
            got.append(bufs[(k - 1) % 2].numpy().copy())   # the previous call's copy has landed
    eng.synchronize()
    got.append(bufs[5 % 2].numpy().copy())
    for k in range(6):
        orc.step(1)
        assert _same(got[k], orc.get_point_positions()), k
    assert _same(got[-1], eng.get_point_positions())
    with pytest.raises(StatusError):          # pageable memory cannot be copied beside the ticks
        eng.enqueue_point_positions_into(np.empty(2 * n, dtype=np.float32))
    import ctypes
    small = bufs[0].numpy()
    with pytest.raises(StatusError):          # a buffer short of 2 floats a point
        eng._call("enqueue_point_positions", small.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 4)
