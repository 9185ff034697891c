"""The allocation-free tick, fse_tick_noalloc, against fse_world_tick.

fse_tick_noalloc is for callers that cannot let the library allocate device
memory (engines that own all device memory through their own arena and budget,
real-time loops that forbid cudaMalloc after start-up). Its scratch is a fixed
array inside the library, so this test hands it plane buffers allocated by torch,
calls it several times in a row, and checks that cells and spawned particles
equal what the ordinary world tick produces, bit for bit: twice on one world,
then on a larger world, then on one with an odd number of chunks per side and
another cell_iter, so that anything a call leaves in the shared scratch and the
next one reads shows up. This file is collected last on purpose, and it passes
alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _Case:
    """One world ticked by fse_world_tick and, on copies of its planes, by
    fse_tick_noalloc."""

    def __init__(self, fse, torch, W, H, cell_iter, seed):
        self.fse, self.W, self.H, self.cell_iter, self.seed = fse, W, H, cell_iter, seed
        self.ref = fse.World(W, H, chunk_size=128, cell_iter=cell_iter, seed=seed)
        self.ref.generate(fse.GEN_MIX, seed)
        host = self.ref.state()
        self.planes = {
            "id": torch.from_numpy(host["id"].view(np.int16).copy()).cuda(),
            "colour": torch.from_numpy(host["colour"].view(np.int32).copy()).cuda(),
            "scalar": torch.from_numpy(host["scalar"].copy()).cuda(),
            "flags": torch.from_numpy(host["flags"].copy()).cuda(),
            "diff": torch.from_numpy(host["diff"].copy()).cuda(),
        }
        self.cap = 40000
        self.out = torch.zeros(self.cap * fse.PARTICLE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        self.tick_no = 0
        self.seen = 0

    def step_and_compare(self, torch):
        fse, L = self.fse, self.fse.lib()
        W, H = self.W, self.H
        n = C.c_int(-1)
        torch.cuda.synchronize()
        ptrs = (C.c_void_p(self.planes[k].data_ptr()) for k in ("id", "colour", "scalar", "flags", "diff"))
        st = L.fse_tick_noalloc(*ptrs, W, H, 128, self.cell_iter, self.seed, self.tick_no,
                                C.c_void_p(self.out.data_ptr()), self.cap, C.byref(n), None)
        assert st == 0, L.fse_status_string(st)
        what = "%dx%d iter %d tick %d" % (W, H, self.cell_iter, self.tick_no)
        self.tick_no += 1
        self.ref.tick(1)
        want = self.ref.state()
        got = {k: self.planes[k].cpu().numpy().view(want[k].dtype).reshape(H, W) for k in self.planes}
        for k in ("id", "colour", "scalar", "flags"):
            np.testing.assert_array_equal(got[k], want[k], err_msg="%s plane %s" % (what, k))
        soup = np.isin(want["id"], [i for i in range(fse.material_count()) if fse.material_get(i)[0] == 3])
        np.testing.assert_array_equal(got["diff"][soup], want["diff"][soup], err_msg="%s diff" % what)
        parts = self.ref.particles()
        new = parts[self.seen:]
        self.seen = len(parts)
        assert n.value == len(new), what
        mine = self.out[: n.value * fse.PARTICLE_DTYPE.itemsize].cpu().numpy().view(fse.PARTICLE_DTYPE)
        # no temperature plane is passed: liquid particles carry temperature 0
        assert not mine["temperature"].any()
        new = new.copy()
        new["temperature"] = 0
        assert mine.tobytes() == new.tobytes(), "%s: spawned particles differ" % what
        return n.value


def test_noalloc_tick_matches_world_tick(fse):
    torch = pytest.importorskip("torch")
    spawned = 0
    first = _Case(fse, torch, 384, 256, 3, 4321)
    for _ in range(2):  # two calls in a row reuse the same scratch
        spawned += first.step_and_compare(torch)
    # a larger world (5 x 4 chunks), then 3 x 3 chunks with two iterations: colours
    # with fewer chunk slots than the largest one, after a call that filled more
    spawned += _Case(fse, torch, 640, 512, 3, 99).step_and_compare(torch)
    spawned += _Case(fse, torch, 384, 384, 2, 7).step_and_compare(torch)
    assert spawned > 0  # the mix spawns free-falling particles, so the comparison is not empty


def test_noalloc_rejects_oversized_requests(fse):
    L = fse.lib()
    n = C.c_int()
    fake = C.c_void_p(16)  # never dereferenced: the size checks come first
    # 16384 x 16384 at chunk 128 needs 4096 chunks of one colour: the limit is 4096
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 16384 + 256, 16384, 128, 3, 0, 0, fake, 0, C.byref(n),
                              None) == -1
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 256, 256, 128, 9, 0, 0, fake, 0, C.byref(n), None) == -1
    assert L.fse_tick_noalloc(fake, fake, fake, fake, fake, 256, 256, 8, 3, 0, 0, fake, 0, C.byref(n), None) == -1
