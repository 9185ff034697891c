"""Shared helpers for the parity tests (compare a device world with the oracle)."""
import numpy as np

SOUP = 3


def soup_mask(ids, mat_types):
    return mat_types[ids] == SOUP


def material_types(fse):
    return np.array([fse.material_get(i)[0] for i in range(fse.material_count())], np.int32)


def compare_states(g, o, types, what=""):
    """Bit-exact comparison of two SoA states; the pending diff only where SOUP."""
    bad = {}
    for k in ("id", "colour", "scalar", "flags"):
        d = int((g[k] != o[k]).sum())
        if d:
            bad[k] = d
    m = types[g["id"]] == SOUP
    d = int((g["diff"][m] != o["diff"][m]).sum())
    if d:
        bad["diff"] = d
    if bad:
        ys, xs = np.nonzero(g["id"] != o["id"]) if "id" in bad else np.nonzero(g[list(bad)[0]] != o[list(bad)[0]])
        where = list(zip(xs[:5].tolist(), ys[:5].tolist()))
        raise AssertionError("%s mismatch %s first cells %s" % (what, bad, where))


def compare_particles(gp, op, what="", temperature=False):
    """Bit-exact comparison of two particle lists. A world that keeps no liquid
    temperatures (created without FSE_CFG_TEMPERATURE) reports 0 where the oracle,
    which always keeps them, has a SOUP tile's temperature: unless `temperature`,
    that field is left out."""
    assert len(gp) == len(op), "%s particle count %d vs %d" % (what, len(gp), len(op))
    if not temperature and len(gp):
        gp, op = gp.copy(), op.copy()
        gp["temperature"] = 0
        op["temperature"] = 0
    if len(gp) and gp.tobytes() != op.tobytes():
        for name in gp.dtype.names:
            d = np.nonzero(gp[name] != op[name])[0]
            if len(d):
                raise AssertionError("%s particle field %s differs at %d entries (first %d: %r vs %r)" % (
                    what, name, len(d), d[0], gp[name][d[0]], op[name][d[0]]))
