"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point that include/*.h declares."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(vg_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def built_lib():
    from vortegrid_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("vg_create", "vg_destroy", "vg_step", "vg_step_device", "vg_get_velocity_grid", "vg_advect",
                 "vg_direct_device", "vg_tree_device", "vg_multigrid_device"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(built_lib, n)]
    assert not missing, missing


def test_python_binding_covers_exports(built_lib):
    import vortegrid_gb300 as vg
    assert set(vg.EXPORTS) <= declared_symbols()
    assert declared_symbols() <= set(vg.EXPORTS)


def test_host_calls_without_gpu(built_lib):
    """Calls that touch no device memory work anywhere."""
    import numpy as np
    import vortegrid_gb300 as vg
    lib = vg.lib()
    assert lib.vg_abi_version() == 2
    cfg = vg.Config()
    assert lib.vg_config_default(ctypes.byref(cfg)) == vg.OK
    assert cfg.poisson_tolerance == 1e-6 and cfg.velocity_technique == vg.VELOCITY_POISSON
    assert lib.vg_status_string(vg.OUT_OF_GRID) == b"out of grid"
    g = vg.define_shape(4096, [-1.5] * 3, [1.5] * 3)
    assert g.points == (17, 17, 17)


def test_define_shape_matches_reference_golden(built_lib, golden):
    """Host-side DefineShape in the library is bit-identical to the reference."""
    import numpy as np
    import vortegrid_gb300 as vg
    for k in range(len(golden["shape_n"])):
        g = vg.define_shape(int(golden["shape_n"][k]), golden["shape_min"][k], golden["shape_max"][k])
        assert np.array_equal(g.as12().view(np.uint32), golden["shape_geom"][k].view(np.uint32)), k
        assert list(g.points) == list(golden["shape_np"][k])


def test_create_fails_cleanly_without_gpu(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import vortegrid_gb300 as vg
    with pytest.raises(vg.VgError) as e:
        vg.Context()
    assert e.value.status == vg.CUDA_ERROR


def test_network_create_fails_cleanly_without_gpu(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import vortegrid_gb300 as vg
    assert vg.lib().vg_net_param_count() == 1472976
    h = ctypes.c_void_p()
    assert vg.lib().vg_net_create(0, None, 128, ctypes.byref(h)) == vg.CUDA_ERROR
    assert not h.value
    assert vg.lib().vg_net_create(0, None, 100, ctypes.byref(h)) == vg.INVALID  # edge/8 must tile
    assert not h.value


def test_invalid_config_rejected(built_lib):
    import vortegrid_gb300 as vg
    cfg = vg.default_config()
    cfg.poisson_tolerance = 0.0
    with pytest.raises(vg.VgError) as e:
        vg.Context(cfg)
    assert e.value.status == vg.INVALID


def test_batch_and_particle_entry_points_reject_bad_arguments(built_lib):
    """Argument checks of the batch solver, team-barrier, wind, kill-age and
    heat-PSE entry points happen before any device call, so they hold
    without a GPU."""
    import vortegrid_gb300 as vg
    L = vg.lib()
    i = ctypes.c_int()
    assert L.vg_batch_set_solver(None, 1, 8, 0) == vg.INVALID
    assert L.vg_batch_solver_info(None, ctypes.byref(i), None, None, None) == vg.INVALID
    for ctas, missing, ms in ((0, 0, 10.0), (4, 5, 10.0), (4, -1, 10.0), (4, 0, 0.0), (4, 0, 20000.0)):
        assert L.vg_team_barrier_check(0, ctas, missing, ms, ctypes.byref(i), ctypes.byref(i)) == vg.INVALID
    wind = (ctypes.c_float * 3)(1.0, 0.0, 0.0)
    assert L.vg_wind_device(None, None, 0, wind, 0.1, 0.9) == vg.INVALID
    m = ctypes.c_size_t()
    assert L.vg_kill_age_device(None, None, None, None, None, 0, 0, 0, ctypes.byref(m)) == vg.INVALID
    g = vg.GridGeom.make([0.0] * 3, [1.0] * 3, [5] * 3)
    assert L.vg_heat_pse_device(None, ctypes.byref(g), None, None, 0, 0.01, 1.0, 0.1) == vg.INVALID
