"""The allocation-free tick, fse_tick_noalloc, against fse_world_tick.

fse_tick_noalloc is for callers that cannot let the library allocate device
memory (engines that own all device memory through their own arena and budget,
real-time loops that forbid cudaMalloc after start-up). Its scratch is a fixed
array inside the library, so this test hands it plane buffers allocated by torch,
calls it twice in a row on the same planes, and checks that cells and spawned
particles equal what the ordinary world tick produces, bit for bit. This file is
collected last on purpose, and it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_tick_matches_world_tick(fse):
    torch = pytest.importorskip("torch")
    L = fse.lib()
    W, H, seed = 384, 256, 4321
    ref = fse.World(W, H, chunk_size=128, cell_iter=3, seed=seed)
    ref.generate(fse.GEN_MIX, seed)
    host = ref.state()
    planes = {
        "id": torch.from_numpy(host["id"].view(np.int16).copy()).cuda(),
        "colour": torch.from_numpy(host["colour"].view(np.int32).copy()).cuda(),
        "scalar": torch.from_numpy(host["scalar"].copy()).cuda(),
        "flags": torch.from_numpy(host["flags"].copy()).cuda(),
        "diff": torch.from_numpy(host["diff"].copy()).cuda(),
    }
    cap = 20000
    out = torch.zeros(cap * fse.PARTICLE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    n = C.c_int(-1)
    torch.cuda.synchronize()
    seen = 0
    for tick in range(2):  # two calls in a row reuse the same scratch
        st = L.fse_tick_noalloc(*(C.c_void_p(planes[k].data_ptr()) for k in ("id", "colour", "scalar", "flags",
                                                                               "diff")),
                                W, H, 128, 3, seed, tick, C.c_void_p(out.data_ptr()), cap, C.byref(n), None)
        assert st == 0, L.fse_status_string(st)
        ref.tick(1)
        want = ref.state()
        got = {k: planes[k].cpu().numpy().view(want[k].dtype).reshape(H, W) for k in planes}
        for k in ("id", "colour", "scalar", "flags"):
            np.testing.assert_array_equal(got[k], want[k], err_msg="tick %d plane %s" % (tick, k))
        soup = np.isin(want["id"], [i for i in range(fse.material_count()) if fse.material_get(i)[0] == 3])
        np.testing.assert_array_equal(got["diff"][soup], want["diff"][soup], err_msg="tick %d diff" % tick)
        parts = ref.particles()
        new = parts[seen:]
        seen = len(parts)
        assert n.value == len(new)
        mine = out[: n.value * fse.PARTICLE_DTYPE.itemsize].cpu().numpy().view(fse.PARTICLE_DTYPE)
        # no temperature plane is passed: liquid particles carry temperature 0
        assert not mine["temperature"].any()
        new = new.copy()
        new["temperature"] = 0
        assert mine.tobytes() == new.tobytes(), "tick %d spawned particles differ" % tick
    assert seen > 0  # the mix spawns free-falling particles, so the comparison is not empty


def test_noalloc_rejects_oversized_requests(fse):
    L = fse.lib()
    n = C.c_int()
    fake = C.c_void_p(16)  # never dereferenced: the size checks come first
    # 16384 x 16384 at chunk 128 needs 4096 chunks of one colour: the limit is 4096
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 16384 + 256, 16384, 128, 3, 0, 0, fake, 0, C.byref(n),
                              None) == -1
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 256, 256, 128, 9, 0, 0, fake, 0, C.byref(n), None) == -1
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 256, 256, 8, 3, 0, 0, fake, 0, C.byref(n), None) == -1
