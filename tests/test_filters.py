"""Contact filtering beyond the fixture definition: b2Fixture.SetFilterData with Refilter
(dynamics/b2fixture.d:132-180) and b2World.SetContactFilter (dynamics/b2world.d:52-55) with a
user b2ContactFilter (b2worldcallbacks.d:47-64), here a class table; the library against the
oracle, which installs the same filter as a b2ContactFilter subclass, bit for bit."""
import numpy as np
import pytest

from compare import exact_diff
from dbox_gb300 import scenes

pytestmark = pytest.mark.gpu

# class 0 meets everything, class 1 meets 0 and 1, class 2 meets class 0 only
TABLE = np.zeros(64, np.uint64)
TABLE[0], TABLE[1], TABLE[2] = 0b111, 0b011, 0b001


def test_table_filter_and_set_filter_data_exact(oracle_lib, gpu_lib):
    oracle_lib.set_trig_mode(1)
    s = scenes.scatter(160, 20.0, 24.0, np.random.default_rng(43))
    nf = len(s["fixtures"])
    ow = oracle_lib.OracleWorld(s)
    gw = gpu_lib.World(s)
    for f in range(4, nf):                              # the container walls keep class 0
        ow.set_filter_class(f, f % 3)
        gw.set_filter_class(0, f, f % 3)
    ow.set_contact_filter(TABLE, True)
    gw.set_contact_filter(0, TABLE, True)

    def check(tag):
        d = exact_diff(ow.export_state(), gw.export_state())
        assert not d, "%s: %s" % (tag, d[:6])

    for t in range(60):
        ow.step()
        gw.step()
        if (t + 1) % 10 == 0:
            check("table filter, step %d" % (t + 1))
    c = gw.export_state()["contacts"]
    cls = lambda f: 0 if f < 4 else f % 3
    pairs = {(cls(a), cls(b)) for a, b in zip(c["fixture_a"], c["fixture_b"])}
    assert not pairs & {(2, 2), (1, 2), (2, 1)}
    # SetFilterData on some fixtures: their contacts are checked again, their proxies touched
    for f in range(5, nf, 11):
        ow.set_filter(f, 0x0002, 0xFFFF & ~0x0002, 0)
        gw.set_filter(0, f, 0x0002, 0xFFFF & ~0x0002, 0)
    for f in range(6, nf, 13):
        ow.set_filter_class(f, 0)
        gw.set_filter_class(0, f, 0)
    check("after SetFilterData")
    for t in range(40):
        ow.step()
        gw.step()
        if (t + 1) % 10 == 0:
            check("refiltered, step %d" % (t + 1))
    # the table alone decides (the default rule off), then the default filter back
    ow.set_contact_filter(TABLE, False)
    gw.set_contact_filter(0, TABLE, False)
    for f in range(7, nf, 17):
        ow.set_filter_class(f, 2)
        gw.set_filter_class(0, f, 2)
    ow.step(steps=30)
    gw.step(steps=30)
    check("table only")
    ow.set_contact_filter(None)
    gw.set_contact_filter(0, None)
    for f in range(4, nf, 5):
        ow.set_filter_class(f, 1)
        gw.set_filter_class(0, f, 1)
    ow.step(steps=30)
    gw.step(steps=30, graph=True)
    check("default filter again")
    bad = TABLE.copy()
    bad[1] = 0b101                                       # row 1 meets class 2, row 2 does not meet 1
    with pytest.raises(gpu_lib.DboxError):
        gw.set_contact_filter(0, bad, True)
