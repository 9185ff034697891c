"""Seeded scenes for pinning rigid-body OBJECT stamping and readback against the
reference's own loops (game.cpp:1766-1813, 1907-1967): a generated mix world and
rotated boxes, some overlapping each other and the world's solids."""
import numpy as np

W, H = 256, 192


def bodies(seed, body_dtype, obj_id, nb=12):
    rng = np.random.default_rng(seed)
    b = np.zeros(nb, body_dtype)
    b["x"] = rng.uniform(30, W - 60, nb).astype(np.float32)
    b["y"] = rng.uniform(30, H - 60, nb).astype(np.float32)
    ang = rng.uniform(0, 6.283, nb).astype(np.float32)
    ang[: nb // 3] = 0.0  # a third axis-aligned
    b["sin_a"] = np.sin(ang).astype(np.float32)
    b["cos_a"] = np.cos(ang).astype(np.float32)
    b["w"] = rng.integers(3, 20, nb)
    b["h"] = rng.integers(3, 20, nb)
    b["id"] = obj_id
    b["colour"] = rng.integers(0, 1 << 24, nb)
    return b


def particle_rows(parts):
    """(id, colour, x, y) of displaced particles as uint32 rows (the reference
    harness's layout); velocities differ by design (rand() there)."""
    return np.stack([parts["id"].astype(np.uint32), parts["colour"].astype(np.uint32),
                     parts["x"].view(np.uint32), parts["y"].view(np.uint32)], 1)
