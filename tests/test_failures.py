"""Failure paths of the step, all made on the host or with a bounded wait (none faults, traps
or hangs the GPU): a contact pool too small for the scene (DBOX_ERR_CAPACITY), a wait budget of
zero polls for the solve kernel's row copies (DBOX_ERR_TIMEOUT, results unchanged), and a
non-finite force (DBOX_ERR_NAN).  The reference's own guards are iteration caps (GJK,
b2distance.d:203; TOI, b2timeofimpact.d:264,274) and b2_maxSubSteps (b2world.d:1164); the
library bounds every device loop the same way and reports the status after the step."""
import numpy as np
import pytest

from compare import exact_diff
from dbox_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_contact_pool_exhaustion_reports_capacity(oracle_lib, gpu_lib):
    # one contact slot per body (+ 64) cannot hold a 210-box pyramid's ~400 contacts
    s = scenes.pyramid()
    gw = gpu_lib.World(s, contacts_per_body=1)
    with pytest.raises(gpu_lib.DboxError) as e:
        for _ in range(5):
            gw.step()
    assert e.value.code == abi.ERR_CAPACITY
    st = gw.export_state()
    assert len(st["contacts"]) <= len(s["bodies"]) + 64
    # the handle stays usable, and a handle with the default pool is unaffected
    gw.step()
    ok = gpu_lib.World(s)
    ok.step(steps=5)
    oracle_lib.set_trig_mode(1)
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=5)
    assert not exact_diff(ow.export_state(), ok.export_state())


def test_wait_budget_reports_timeout_and_keeps_results(oracle_lib, gpu_lib):
    # with a budget of zero polls every row-copy wait of the solve kernel is reported; the waits
    # still end when their copies land, so the step's results are the oracle's, bit for bit
    oracle_lib.set_trig_mode(1)
    s = scenes.pyramid(rows=12)
    gw = gpu_lib.World(s)
    ow = oracle_lib.OracleWorld(s)
    gw.step(steps=10)
    ow.step(steps=10)
    gw.set_wait_limit(0)
    for _ in range(3):
        with pytest.raises(gpu_lib.DboxError) as e:
            gw.step()
        assert e.value.code == abi.ERR_TIMEOUT
        ow.step()
        assert not exact_diff(ow.export_state(), gw.export_state())
    with pytest.raises(gpu_lib.DboxError) as e:   # the graph path reports it too
        gw.step(steps=4, graph=True)
    assert e.value.code == abi.ERR_TIMEOUT
    ow.step(steps=4)
    gw.set_wait_limit()
    gw.step(steps=10)
    gw.step(steps=10, graph=True)
    ow.step(steps=20)
    assert not exact_diff(ow.export_state(), gw.export_state())


def test_nonfinite_force_reports_nan(gpu_lib):
    # hello_world's box, free in the air, gets a NaN force: its velocity and position leave
    # the finite range in the step's integration and the step reports DBOX_ERR_NAN
    s = scenes.hello_world()
    gw = gpu_lib.World([s, scenes.hello_world()])
    gw.step(steps=2)
    f = np.zeros((4, 3), np.float32)
    f[1, 0] = np.nan                                  # world 0, body 1 (the box)
    gw.apply_forces(f)
    with pytest.raises(gpu_lib.DboxError) as e:
        gw.step()
    assert e.value.code == abi.ERR_NAN
    b = gw.bodies()
    assert not np.isfinite(b["position"][1]).all()
    assert np.isfinite(b["position"][3]).all()        # the other world is untouched
