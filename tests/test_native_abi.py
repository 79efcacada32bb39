"""CPU checks of the C ABI boundary: the library loads and exports every
function include/sailor_gb300.h declares; host-side argument validation
raises before any kernel launch.  No compute call is made without a GPU."""
import ctypes as C
import os
import re

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    src = open(os.path.join(ROOT, "include", "sailor_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from sailor_gb300 import build
    path = build.build_library()
    return C.CDLL(path)


def test_header_symbols_exported(lib):
    names = _header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from sailor_gb300 import _native as N
    assert set(_header_functions()) <= set(N.EXPORTS)


def test_status_strings_and_constants(lib):
    lib.sg_status_string.restype = C.c_char_p
    for code in range(5):
        assert lib.sg_status_string(code)
    assert lib.sg_status_string(0) == b"ok"
    assert lib.sg_mask_words(2) == 1 and lib.sg_mask_words(4) == 2 and lib.sg_mask_words(8) == 16
    lib.sg_tree_scratch_bytes.restype = C.c_size_t
    assert lib.sg_tree_scratch_bytes(1, 32) >= 2 * 4 * 32 ** 3


def test_det_counter_indices_match_header(tmp_path):
    """The Python mirror of the reduction workspace's counter indices has
    the header's values (a probe compiled with gcc against the header)."""
    import shutil
    import subprocess
    from sailor_gb300 import _native as N
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    names = ["SG_DET_COUNTERS", "SG_DET_RAYS_WITH_HITS", "SG_DET_SLOTS_NEEDED", "SG_DET_SLOTS", "SG_DET_CELLS",
             "SG_DET_RECORDS", "SG_FLAG_HIT_OVERFLOW", "SG_FLAG_TREE_CAPACITY", "SG_FLAG_RECORD_CAPACITY"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(['#include <stdio.h>', '#include "sailor_gb300.h"', "int main(void) {"] +
                             [f'  printf("{n} %d\\n", (int)({n}));' for n in names] + ["  return 0;", "}"]))
    exe = tmp_path / "probe"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call(["gcc", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)])
    for line in subprocess.check_output([str(exe)]).decode().splitlines():
        n, v = line.split()
        assert getattr(N, n) == int(v), n


def test_null_arguments_rejected(lib):
    """Entry points validate pointers and sizes before launching."""
    from sailor_gb300 import _native as N
    L = N.lib
    assert L.sg_fuse_tsdf(*([None] * 4), 1, 1, 8, 8, 8, 8, 8, None, None, 1.0, 3.0, 13.5, 13.5,
                          *([None] * 5), None) == 1
    assert L.sg_sort_samples(None, 1, 8, None, None, None) == 1
    assert L.sg_composite_fwd(None, None, None, None, 1, 8, 3, 1e-4, 0, None, None, None, None, None) == 1
    assert L.sg_brick_occupancy(None, 1, 8, 4, None, None, None) == 1


def test_cpu_tensors_rejected():
    from sailor_gb300.dist import VoxelEncoding as VE
    z = torch.zeros(1, 4, 8)
    with pytest.raises(RuntimeError, match="cuda"):
        VE.volume_rendering_occ_forward(z, torch.zeros(1, 4, 8, 1), torch.zeros(1, 4, 8, 3), 0, 1e-4)
    with pytest.raises(RuntimeError, match="cuda"):
        VE.build_multi_res_volumes([torch.zeros(1, 8, 8, 8, dtype=torch.int32)], [torch.zeros(1, 1)], 2, 4, 0)


def test_unsupported_tree_shapes():
    """Depths outside [2, SG_MAX_LEVELS] and rates other than 2, 4, 8 are
    refused on the host before anything reaches the device; the traversal
    and fine sampling refuse to run before init_octree."""
    from sailor_gb300 import _native as N
    from sailor_gb300.dist import VoxelEncoding as VE
    o = VE.MultiLayerOctree(1, 1, 2, 0)
    with pytest.raises(RuntimeError, match="levels"):
        o.init_octree([None], [0], [None], [0], None, None)
    o = VE.MultiLayerOctree(N.SG_MAX_LEVELS + 1, 1, 2, 0)
    with pytest.raises(RuntimeError, match="levels"):
        o.init_octree([None] * (N.SG_MAX_LEVELS + 1), [0] * 13, [None] * 13, [0] * 13, None, None)
    o = VE.MultiLayerOctree(3, 1, 3, 0)
    with pytest.raises(RuntimeError, match="rate"):
        o.init_octree([None] * 3, [0, 0, 0], [None] * 3, [0, 0, 0], None, None)
    o = VE.MultiLayerOctree(3, 1, 2, 0)
    with pytest.raises(RuntimeError, match="before init_octree"):
        o.octree_traversal(None, None, 8, 8, 0, -1, -1)
    with pytest.raises(RuntimeError, match="before init_octree"):
        o.ray_voxels_points_sampling(None, None, None, None, None, 0, 8)


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror of a header struct has the C compiler's size and
    field offsets (a probe compiled with gcc against the header)."""
    import shutil
    import subprocess
    from sailor_gb300 import _native as N
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    structs = {name: getattr(N, name) for name in ("SgTree", "SgViews", "SgRaySegments", "SgRenderArgs",
                                                   "SgFeatureMap", "SgProjGather", "SgOctree")}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sailor_gb300.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{name} {fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call(["gcc", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)]).decode().splitlines():
        name, field, val = line.split()
        got[(name, field)] = int(val)
    for name, cls in structs.items():
        assert got[(name, "size")] == C.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert got[(name, fname)] == getattr(cls, fname).offset, (name, fname)
