"""GPU parity of the remaining hot-path features against the CPU oracle: fire and
reactions, material interactions (wide halo), scripted materials, free particles
(bit-exact FP32 and within 1e-5 of FP64), CUDA-graph replay, batches, the
autotuner, rigid OBJECT stamping/readback/export and the serving loop."""
import numpy as np
import pytest

from helpers import compare_particles, compare_states, material_types

pytestmark = pytest.mark.gpu
PART = 1


def _pair(fse, oracle_mod, w, h, seed, kind=1):
    world = fse.World(w, h, chunk_size=128, cell_iter=3, seed=seed)
    world.generate(kind, seed)
    ow = oracle_mod.OracleWorld(w, h, 128, 3, seed)
    ow.generate({1: 0, 2: 1}[kind], seed)
    return world, ow


def _sprinkle(fse, state, seed, specs):
    rng = np.random.default_rng(seed)
    for name, frac, scalar in specs:
        m = fse.material_find(name)
        pick = rng.random(state["id"].shape) < frac
        state["id"][pick] = m
        state["scalar"][pick] = scalar
        state["colour"][pick] = 0x00ABCDEF
        state["flags"][pick] = 0
        state["diff"][pick] = 0
    return state


def _run_both(fse, oracle_mod, world, ow, steps, what):
    types = material_types(fse)
    for t in range(steps):
        world.step(1)
        ow.step(1, PART)
        compare_states(world.state(), ow.state(), types, "%s step %d" % (what, t))
        compare_particles(world.particles(), ow.particles(), "%s step %d" % (what, t))


def test_fire_lava_steam_reactions(fse, oracle_mod):
    world, ow = _pair(fse, oracle_mod, 256, 192, 31)
    s = _sprinkle(fse, world.state(), 3, [("FIRE", 0.02, 0), ("LAVA", 0.03, 2 * 65536), ("STEAM", 0.03, 0),
                                           ("GOLD_ORE", 0.02, 600), ("COBBLE_STONE", 0.05, 0)])
    world.upload(s)
    ow.set_state(s)
    _run_both(fse, oracle_mod, world, ow, 6, "fire")
    np.testing.assert_array_equal(world.ledger(), ow.ledger())


def test_interactions_use_the_wide_halo(fse, oracle_mod):
    o = oracle_mod.Oracle()
    sand, dirt, water, stone, cobble = (fse.material_find(n) for n in ("GENERIC_SAND", "DIRT", "WATER", "STONE",
                                                                       "COBBLE_STONE"))
    # boxes reaching 5 cells to the side and below; the last one has a negative low
    # corner, which the reference's unsigned loop bound never visits
    rules = [(sand, water, 1, dirt, 2, 3, 2), (sand, stone, 2, water, 1, 1, 4), (sand, cobble, 2, water, 1, -2, 0)]
    try:
        for r in rules:
            fse.set_interaction(*r)
            assert o.set_interaction(*r) == 0
        fse.PushMaterials()
        world, ow = _pair(fse, oracle_mod, 256, 256, 8)
        _run_both(fse, oracle_mod, world, ow, 4, "interactions")
    finally:
        fse.InitMaterials()
        fse.PushMaterials()
        o.reset_materials()


def test_lua_registered_material(fse, oracle_mod):
    o = oracle_mod.Oracle()
    script = """
    -- materials registered from a script, as data/scripts would
    materials_register(2001, "Heavy Sand", "HEAVY_SAND", 2, 12, 255, 30.5, 2, 0, 0, 0xFFAA3300)
    materials_register(2002, 'Oil', 'OIL', 3, 0, 0x80, 0.8, 5, 0, 0, 0xFF202020)
    """
    try:
        assert fse.load_lua_materials(script) == 2
        hs = o.register(2001, "Heavy Sand", "HEAVY_SAND", 2, 12, 255, 30.5, 2, 0, 0, 0xFFAA3300)
        oil = o.register(2002, "Oil", "OIL", 3, 0, 0x80, 0.8, 5, 0, 0, 0xFF202020)
        assert (hs, oil) == (fse.material_find("HEAVY_SAND"), fse.material_find("OIL"))
        for i in range(fse.material_count()):
            np.testing.assert_array_equal(fse.material_get(i), o.material(i))
        fse.PushMaterials()
        world, ow = _pair(fse, oracle_mod, 192, 192, 12)
        s = _sprinkle(fse, world.state(), 5, [("HEAVY_SAND", 0.1, 0), ("OIL", 0.1, 65536)])
        world.upload(s)
        ow.set_state(s)
        _run_both(fse, oracle_mod, world, ow, 5, "lua")
    finally:
        fse.InitMaterials()
        fse.PushMaterials()
        o.reset_materials()


def _particles(fse, n, w, h, seed, temporary=False):
    rng = np.random.default_rng(seed)
    p = np.zeros(n, fse.PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, w, n).astype(np.float32)
    p["y"] = rng.uniform(0, h, n).astype(np.float32)
    p["vx"] = rng.normal(0, 2, n).astype(np.float32)
    p["vy"] = rng.normal(0, 2, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    p["id"] = fse.material_find("GENERIC_SAND")
    p["colour"] = 0xFFFFFFFF
    if temporary:
        p["bits"][::7] = 2
        p["lifetime"][::7] = rng.integers(0, 5, len(p["lifetime"][::7]))
    return p


def test_free_particles_bit_exact(fse, oracle_mod):
    world, ow = _pair(fse, oracle_mod, 512, 384, 77)
    p = _particles(fse, 40000, 512, 384, 1, temporary=True)
    water = fse.material_find("WATER")
    p["id"][1::5] = water
    p["scalar"][1::5] = 65536 * 3
    world.addCell(p)
    ow.set_particles(p)
    _run_both(fse, oracle_mod, world, ow, 6, "particles")


def test_particles_within_1e5_of_fp64(fse, oracle_mod):
    """One tickCells() of free-flying particles vs the FP64 kinematics oracle."""
    world = fse.World(512, 512, seed=3)  # an empty world: no collisions
    ow = oracle_mod.OracleWorld(512, 512, 128, 3, 3)
    p = _particles(fse, 20000, 512, 512, 9)
    p["x"] = np.clip(p["x"], 64, 448)
    p["y"] = np.clip(p["y"], 64, 448)
    world.addCell(p)
    world.tickCells()
    g = world.particles()
    ref, ev, _ = ow.kinematics(p, f64=True)
    alive = ev == 0
    assert alive.sum() == len(g)
    ref = ref[alive]
    got = np.stack([g["x"], g["y"], g["vx"], g["vy"]], 1).astype(np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
    assert rel.max() <= 1e-5, rel.max()


def test_graph_replay_equals_plain_steps(fse):
    a = fse.World(384, 256, seed=5)
    b = fse.World(384, 256, seed=5)
    a.generate(fse.GEN_MIX, 5)
    b.generate(fse.GEN_MIX, 5)
    a.step(40)
    b.step(40, graph=True)
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    assert a.particles().tobytes() == b.particles().tobytes()
    assert a.tick_count == b.tick_count == 40


def test_batch_equals_individual_worlds(fse):
    sizes = [(128, 192), (320, 128), (256, 256), (192, 448), (512, 320)]
    solo = []
    for i, (w, h) in enumerate(sizes):
        x = fse.World(w, h, seed=100 + i)
        x.generate(fse.GEN_MIX, 100 + i)
        x.step(9)
        solo.append(x)
    worlds = []
    for i, (w, h) in enumerate(sizes):
        x = fse.World(w, h, seed=100 + i)
        x.generate(fse.GEN_MIX, 100 + i)
        worlds.append(x)
    b = fse.Batch(worlds)
    b.step(4)
    b.step(5, graph_ticks=3)
    for x, y in zip(solo, worlds):
        sx, sy = x.state(), y.state()
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=k)
        assert x.particles().tobytes() == y.particles().tobytes()
    b.close()


def _free_particles(fse, n, w, h, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(n, fse.PARTICLE_DTYPE)
    p["x"] = rng.uniform(0, w, n).astype(np.float32)
    p["y"] = rng.uniform(-8, h + 24, n).astype(np.float32)  # some start below the world
    p["vx"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["vy"] = rng.normal(0.0, 2.0, n).astype(np.float32)
    p["ay"] = np.float32(0.1)
    p["fade_time"] = 60
    p["id"] = fse.material_find("GENERIC_SAND")
    p["colour"] = 0xFFFFFFFF
    return p


def test_batch_compaction_across_uneven_particle_lists(fse):
    """The particle-list compaction runs over one index space of every world's
    particles: worlds with no particles at all, with tens of thousands, and with
    particles leaving through the bottom, side by side, equal the same worlds alone."""
    specs = [(256, 192, fse.GEN_EMPTY, 0), (384, 320, fse.GEN_MIX, 20000), (128, 128, fse.GEN_EMPTY, 0),
             (320, 256, fse.GEN_MIX, 3000), (192, 448, fse.GEN_EMPTY, 700)]
    solo, worlds = [], []
    for i, (w, h, kind, n) in enumerate(specs):
        for lst in (solo, worlds):
            x = fse.World(w, h, seed=500 + i)
            x.generate(kind, 500 + i)
            if n:
                x.addCell(_free_particles(fse, n, w, h, 500 + i))
            lst.append(x)
    for x in solo:
        x.step(5)
    b = fse.Batch(worlds)
    b.step(5)
    assert worlds[0].particle_count() == 0 and worlds[2].particle_count() == 0
    for x, y in zip(solo, worlds):
        sx, sy = x.state(), y.state()
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=k)
        assert x.particles().tobytes() == y.particles().tobytes()
    b.close()


def test_disjoint_batches_enqueued_concurrently(fse):
    """Two batches of disjoint worlds enqueued on their own streams without waiting
    (fused ticks and cooperative particle updates of both in flight together), with
    whole-batch plane I/O between steps as a pipelined round trip does: every world
    equals the same world stepped alone."""
    sizes = [(128, 192), (320, 128), (256, 256), (192, 448), (512, 320), (384, 384)]
    solo, worlds = [], []
    for i, (w, h) in enumerate(sizes):
        for lst in (solo, worlds):
            x = fse.World(w, h, seed=300 + i)
            x.generate(fse.GEN_MIX, 300 + i)
            lst.append(x)
    for x in solo:
        x.step(7)
    torch = pytest.importorskip("torch")
    groups = [fse.Batch(worlds[:3]), fse.Batch(worlds[3:])]
    bufs = [torch.empty(g.io_layout()[1], dtype=torch.uint8, pin_memory=True).numpy() for g in groups]
    for g, buf in zip(groups, bufs):
        g.download_all(buf)
    for g in groups:
        g.sync()
    for n in (4, 3):
        for g, buf in zip(groups, bufs):
            g.upload_all(buf)
            g.enqueue(n)
            g.download_all(buf)
        for g in groups:
            g.sync()
    views = groups[0].io_views(bufs[0]) + groups[1].io_views(bufs[1])
    for x, y, v in zip(solo, worlds, views):
        sx, sy = x.state(), y.state()
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=k)
            np.testing.assert_array_equal(sx[k], v[k], err_msg="downloaded " + k)
        assert x.particles().tobytes() == y.particles().tobytes()
    for g in groups:
        g.close()


def test_autotune_never_changes_results(fse):
    ref = fse.World(384, 384, seed=44)
    ref.generate(fse.GEN_MIX, 44)
    ref.step(11)
    w = fse.World(384, 384, seed=44)
    w.generate(fse.GEN_MIX, 44)
    b = fse.Batch([w])
    choice = b.autotune()
    assert choice["colour_ctas_per_sm"] in (0, 1, 2, 3, 4) and choice["particle_blocks"] >= 0
    assert w.tick_count == 0  # the autotuner restored the world
    b.step(3)
    # every launch shape gives the same world
    for shape in ((1, 4), (0, 1), (4, 0), (1, 0), (2, 0), (3, 4), (4, 16), (2, 16)):
        b.set_launch(*shape)
        b.step(1)
    sr, sw = ref.state(), w.state()
    for k in sr:
        np.testing.assert_array_equal(sr[k], sw[k], err_msg=k)
    b.close()


def _boxes(fse, n, w, h, seed):
    rng = np.random.default_rng(seed)
    b = np.zeros(n, fse.BODY_DTYPE)
    b["w"] = rng.integers(8, 65, n)
    b["h"] = rng.integers(8, 65, n)
    b["x"] = rng.uniform(0, w - 8, n).astype(np.float32)
    b["y"] = rng.uniform(0, h - 8, n).astype(np.float32)
    b["cos_a"] = 1.0
    b["id"] = fse.material_find("GENERIC_OBJECT")
    b["colour"] = 0xFF00FF00
    return b


def test_object_stamp_readback_and_mask(fse, oracle_mod):
    types = material_types(fse)
    world, ow = _pair(fse, oracle_mod, 512, 512, 9, kind=2)
    bodies = _boxes(fse, 30, 512, 512, 4)
    # one rotated body as well
    bodies[0]["sin_a"], bodies[0]["cos_a"] = np.float32(np.sin(0.5)), np.float32(np.cos(0.5))
    ob = bodies.copy()
    for t in range(3):
        world.object_stamp(bodies)
        ow.object_stamp(ob)
        for f in ("n_sand", "n_soup", "n_placed"):
            np.testing.assert_array_equal(bodies[f], ob[f], err_msg=f)
        compare_states(world.state(), ow.state(), types, "stamp %d" % t)
        compare_particles(world.particles(), ow.particles(), "stamp %d" % t)
        world.step(1)
        ow.step(1, PART)
        np.testing.assert_array_equal(world.object_mask(), ow.object_mask())
        lst, n = world.object_list()
        bits = np.unpackbits(ow.object_mask(), bitorder="little")[: 512 * 512]
        np.testing.assert_array_equal(lst, np.nonzero(bits)[0].astype(np.uint32))
        assert n == len(lst)
        rg = world.object_readback(bodies)
        ro = ow.object_readback(ob)
        assert rg == ro
        np.testing.assert_array_equal(bodies["n_recovered"], ob["n_recovered"])
        compare_states(world.state(), ow.state(), types, "readback %d" % t)


def test_serving_alone_equals_in_the_mix(fse):
    sizes = [(256, 256), (384, 256), (256, 512)]
    srv = fse.Server(8 << 30, max_active=8)
    slots = [srv.add_world(w, h, fse.GEN_MIX, 500 + i, seed=500 + i) for i, (w, h) in enumerate(sizes)]
    reqs = [(slots[0], 5), (slots[1], 3), (slots[2], 7), (slots[0], 2), (slots[1], 4)]
    for s, n in reqs:
        srv.submit(s, n)
    done = 0
    for _ in range(200):
        srv.step()
        ids, _ = srv.poll()
        done += len(ids)
        if done == len(reqs):
            break
    assert done == len(reqs)
    ticks = {slots[0]: 7, slots[1]: 7, slots[2]: 7}
    for i, (w, h) in enumerate(sizes):
        alone = fse.World(w, h, seed=500 + i)
        alone.generate(fse.GEN_MIX, 500 + i)
        alone.step(ticks[slots[i]])
        mixed = srv.world(slots[i])
        sa, sm = alone.state(), mixed.state()
        for k in sa:
            np.testing.assert_array_equal(sa[k], sm[k], err_msg="world %d %s" % (i, k))
        assert alone.particles().tobytes() == mixed.particles().tobytes()
    srv.close()


def test_batch_async_plane_io(fse):
    """fse_batch_upload / fse_batch_download on the batch's stream: a round trip of
    planes between steps equals the world API; an out-of-range id becomes AIR and
    the next sync reports it once."""
    sizes = [(256, 200), (384, 256)]
    worlds = [fse.World(w, h, seed=60 + i) for i, (w, h) in enumerate(sizes)]
    twins = [fse.World(w, h, seed=60 + i) for i, (w, h) in enumerate(sizes)]
    for i, (a, b) in enumerate(zip(worlds, twins)):
        a.generate(fse.GEN_MIX, 60 + i)
        b.generate(fse.GEN_MIX, 60 + i)
    batch = fse.Batch(worlds)
    host = [w.state() for w in twins]
    for k, st in enumerate(host):
        st["id"][:8, :8] = fse.material_find("WATER")
        batch.upload(k, st)
        twins[k].upload(st)
    batch.step(2)
    out = [{k: np.empty_like(v) for k, v in st.items()} for st in host]
    for k in range(len(worlds)):
        batch.download(k, out[k])
    batch.sync()
    for k, tw in enumerate(twins):
        tw.step(2)
        ref = tw.state()
        for key in ref:
            np.testing.assert_array_equal(out[k][key], ref[key], err_msg="world %d %s" % (k, key))
    bad = dict(out[0])
    bad["id"] = bad["id"].copy()
    bad["id"][0, 0] = 999
    batch.upload(0, bad)
    with pytest.raises(fse.FseError):
        batch.sync()
    assert worlds[0].state()["id"][0, 0] == fse.material_find("GENERIC_AIR")
    batch.sync()  # reported once
    # the whole batch through one buffer
    offs, total = batch.io_layout()
    assert offs[0, 0] == 0 and total % 16 == 0 and np.all(offs % 16 == 0)
    buf = np.zeros(total, np.uint8)
    batch.download_all(buf)
    batch.sync()
    views = batch.io_views(buf)
    for k, w in enumerate(worlds):
        ref = w.state()
        for key in ref:
            np.testing.assert_array_equal(views[k][key], ref[key], err_msg="download_all %d %s" % (k, key))
    for k, tw in enumerate(twins):
        for key, v in tw.state().items():
            views[k][key][...] = v
    views[1]["flags"][...] |= 0x40  # the visited bit is cleared on upload
    batch.upload_all(buf)
    batch.step(1)
    batch.sync()
    for k, tw in enumerate(twins):
        tw.step(1)
        a, b = worlds[k].state(), tw.state()
        for key in a:
            np.testing.assert_array_equal(a[key], b[key], err_msg="upload_all %d %s" % (k, key))
    views[1]["id"][3, 5] = 1000
    batch.upload_all(buf)
    with pytest.raises(fse.FseError):
        batch.sync()
    batch.close()
    for w in worlds + twins:
        w.close()


def test_serving_parks_worlds_beyond_the_budget(fse):
    """Four worlds under a budget that holds two: requests for parked worlds are
    admitted by parking idle ones; every world ends as if ticked alone."""
    sizes = [(256, 256), (384, 256), (256, 512), (320, 320)]
    probe = fse.Server(8 << 30, max_active=4)
    foot = []
    for i, (w, h) in enumerate(sizes):
        before = probe.bytes_in_use()
        probe.add_world(w, h, fse.GEN_MIX, 700 + i, seed=700 + i)
        foot.append(probe.bytes_in_use() - before)
    probe.close()
    budget = int(2.3 * max(foot))
    srv = fse.Server(budget, max_active=2)
    srv.set_depth(4)
    slots = [srv.add_world(w, h, fse.GEN_MIX, 700 + i, seed=700 + i) for i, (w, h) in enumerate(sizes)]
    assert srv.bytes_in_use() <= budget
    assert srv.stats()["parked"] >= 1
    reqs = [(0, 3), (2, 2), (1, 4), (3, 1), (0, 2), (3, 3), (2, 1), (1, 1), (0, 1)]
    t_sub = {}
    for k, n in reqs:
        t_sub[srv.submit(slots[k], n)] = srv.now_us()
    got = {}
    for _ in range(400):
        srv.step()
        assert srv.bytes_in_use() <= budget
        ids, t_done = srv.poll()
        got.update(zip(ids.tolist(), t_done.tolist()))
        if len(got) == len(reqs):
            break
    assert len(got) == len(reqs)
    for rid, td in got.items():
        assert td >= t_sub[rid] - 50.0  # device completion after the submit (clock anchor slack)
    st = srv.stats()
    assert st["restored"] >= 1 and st["parked_out"] >= 1
    assert len(srv.tick_times()) == st["steps"]
    ticks = [0] * len(sizes)
    for k, n in reqs:
        ticks[k] += n
    for i, (w, h) in enumerate(sizes):
        alone = fse.World(w, h, seed=700 + i)
        alone.generate(fse.GEN_MIX, 700 + i)
        alone.step(ticks[i])
        served = srv.world(slots[i])
        assert served is not None and srv.bytes_in_use() <= budget
        sa, sm = alone.state(), served.state()
        for key in sa:
            np.testing.assert_array_equal(sa[key], sm[key], err_msg="world %d %s" % (i, key))
        assert alone.particles().tobytes() == served.particles().tobytes()
        assert alone.tick_count == served.tick_count
    srv.close()


def test_serving_admission_respects_the_budget(fse):
    srv = fse.Server(64 << 20, max_active=4)
    assert srv.try_add_world(256, 256) is not None
    assert srv.try_add_world(4096, 4096) is None  # refused by the HBM budget
    assert srv.bytes_in_use() <= 64 << 20
    srv.close()


def test_world_api_roundtrip(fse):
    w = fse.World(200, 136, seed=1)
    w.generate(fse.GEN_MIX, 1)
    s = w.state()
    t = w.getTile(5, 7)
    assert (t.id, t.colour) == (int(s["id"][7, 5]), int(s["colour"][7, 5]))
    assert w.getTile(-1, 0).id == fse.material_find("GENERIC_SOLID")  # world.cpp:1000
    w.setTile(5, 7, fse.MaterialInstance(fse.material_find("WATER"), 0x1234, 65536, 0))
    w.setTile(500, 7, fse.MaterialInstance(1))  # dropped, world.cpp:1005
    assert w.getTile(5, 7).scalar == 65536
    w.tick_count = 17
    assert w.tick_count == 17
    bad = dict(s)
    bad["id"] = np.full_like(s["id"], 999)
    with pytest.raises(fse.FseError):
        w.upload(bad)
