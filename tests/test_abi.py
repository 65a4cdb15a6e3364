"""CPU checks of the C-ABI boundary: the library builds and loads, exports every
function include/dbox_gpu.h declares, and its record layouts match the numpy
mirrors in dbox_gb300/abi.py.  No device computation runs here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from dbox_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dbox_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dbox_[a-z0-9_]+)\s*\(", text)) - {"dbox_event_fn"})


def test_library_exports_every_declared_symbol(gpu_lib):
    L = gpu_lib.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_record_layouts_match_header(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "dbox_gpu.h"\nint main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(dbox_body_def), sizeof(dbox_shape_def), sizeof(dbox_fixture_def), sizeof(dbox_revolute_def),'
                   'sizeof(dbox_world_header), sizeof(dbox_body_state), sizeof(dbox_proxy_state), sizeof(dbox_contact_state),'
                   'sizeof(dbox_joint_state), sizeof(dbox_contact_event), offsetof(dbox_contact_state, points),'
                   'offsetof(dbox_body_state, vel));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [abi.BODY_DEF.itemsize, abi.SHAPE_DEF.itemsize, abi.FIXTURE_DEF.itemsize, abi.REVOLUTE_DEF.itemsize,
            abi.WORLD_HEADER.itemsize, abi.BODY_STATE.itemsize, abi.PROXY_STATE.itemsize, abi.CONTACT_STATE.itemsize,
            abi.JOINT_STATE.itemsize, abi.CONTACT_EVENT.itemsize, abi.CONTACT_STATE.fields["points"][1],
            abi.BODY_STATE.fields["vel"][1]]
    assert got == want


def test_defaults_match_reference(gpu_lib):
    L = gpu_lib.lib()
    b = np.zeros(1, abi.BODY_DEF)
    L.dbox_body_def_default(abi.ptr(b))
    assert b[0]["type"] == abi.STATIC and b[0]["allow_sleep"] == 1 and b[0]["awake"] == 1
    assert b[0]["active"] == 1 and b[0]["gravity_scale"] == np.float32(1.0)
    f = np.zeros(1, abi.FIXTURE_DEF)
    L.dbox_fixture_def_default(abi.ptr(f))
    assert f[0]["friction"] == np.float32(0.2) and f[0]["mask_bits"] == 0xFFFF and f[0]["category_bits"] == 1
    assert (abi.body_defs(1) == b).all() and (abi.fixture_defs(1) == f).all()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_world_create_without_gpu_fails_loudly(gpu_lib):
    from dbox_gb300 import scenes
    with pytest.raises(gpu_lib.DboxError):
        gpu_lib.World(scenes.hello_world())


def test_invalid_arguments_rejected_without_device(gpu_lib):
    L = gpu_lib.lib()
    out = ctypes.c_void_p()
    assert L.dbox_world_create(abi.Vec2(0.0, -10.0), 0, None, ctypes.byref(out)) == -1
    assert L.dbox_world_destroy(None) == -1
    assert L.dbox_world_step(None, ctypes.c_float(0.016), 8, 3) == -1
    assert L.dbox_world_set_wait_limit(None, 0) == -1
    assert L.dbox_world_set_island_solver(None, 0) == -1
    assert L.dbox_world_get_island_solver(None, None) == -1
    assert L.dbox_world_set_fused_step(None, 1) == -1
    assert L.dbox_world_get_fused_step(None, None) == -1
