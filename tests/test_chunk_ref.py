"""The .pack files against the reference's own Chunk::ChunkWrite / ChunkRead.

oracle/Makefile `ref` compiles both functions (source/engine/chunk.cpp:68-330)
unchanged with MaterialInstanceData and the reference's vendored LZ4
(oracle/ref_chunk.cpp). Files written by the reference are read by the oracle's
unpack to the same materials, colours, temperatures and phase; files written by the
oracle's pack (byte for byte the device's, tests/test_gpu_pack.py) are read by the
reference's ChunkRead to the world they came from.
"""
import ctypes as C
import os

import numpy as np
import pytest

from pack_cases import sample_world


def _lib():
    from oracle.binding import HERE, REFERENCE_WORLD_CPP, make_ref

    if not os.path.exists(REFERENCE_WORLD_CPP):
        pytest.skip("reference tree absent")

    make_ref()
    lib = C.CDLL(os.path.join(HERE, "_ref", "libref_chunk.so"))
    lib.ref_chunk_write.argtypes = [C.c_char_p, C.c_int] + [C.c_void_p] * 3
    lib.ref_chunk_read.argtypes = [C.c_char_p] + [C.c_void_p] * 4
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("seed", [3, 4])
def test_pack_files_match_the_reference_chunk_io(oracle_mod, tmp_path, seed):
    lib = _lib()
    oracle_mod.Oracle().reset_materials()
    w, h = 256, 256
    ow = sample_world(oracle_mod, w, h, seed)
    st, temps = ow.state(), ow.temperature()
    ncx = w // 128
    # the reference writes, the oracle reads
    files, offs = [], [0]
    for k in range((w // 128) * (h // 128)):
        cx, cy = k % ncx, k // ncx
        sl = (slice(cy * 128, cy * 128 + 128), slice(cx * 128, cx * 128 + 128))
        path = str(tmp_path / ("c_%d_%d.pack" % (cx, cy)))
        assert lib.ref_chunk_write(path.encode(), 5, _p(np.ascontiguousarray(st["id"][sl])),
                                   _p(np.ascontiguousarray(st["colour"][sl])),
                                   _p(np.ascontiguousarray(temps[sl]))) == 0
        data = np.fromfile(path, np.uint8)
        files.append(data)
        offs.append(offs[-1] + len(data))
    ob = oracle_mod.OracleWorld(w, h, 128, 3, 1)
    rc, phases = ob.unpack(np.concatenate(files), np.array(offs, np.int64))
    assert rc == 0 and np.all(phases == 5)
    got = ob.state()
    assert np.array_equal(got["id"], st["id"]) and np.array_equal(got["colour"], st["colour"])
    assert np.array_equal(ob.temperature(), temps)
    # the oracle writes, the reference reads
    data, offs = ow.pack(-2)
    ids = np.zeros(128 * 128, np.uint16)
    cols = np.zeros(128 * 128, np.uint32)
    tt = np.zeros(128 * 128, np.int16)
    ph = C.c_int(0)
    for k in range(len(offs) - 1):
        cx, cy = k % ncx, k // ncx
        sl = (slice(cy * 128, cy * 128 + 128), slice(cx * 128, cx * 128 + 128))
        path = str(tmp_path / ("o_%d.pack" % k))
        data[offs[k]:offs[k + 1]].tofile(path)
        assert lib.ref_chunk_read(path.encode(), _p(ids), _p(cols), _p(tt), C.byref(ph)) == 0
        assert ph.value == -2
        assert np.array_equal(ids.reshape(128, 128), st["id"][sl]), k
        assert np.array_equal(cols.reshape(128, 128), st["colour"][sl]), k
        assert np.array_equal(tt.reshape(128, 128), temps[sl]), k
