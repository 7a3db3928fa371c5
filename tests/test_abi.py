"""librtg.so loads and exports every entry point include/rtg.h declares; the
ctypes structures match the C layout (no compute calls: runs without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rtg.h")


def _declared():
    text = open(HEADER).read()
    return re.findall(r"^RTG_API\s+[\w\s\*]*?\b(rtg_\w+)\s*\(", text, flags=re.M)


def test_every_declared_symbol_is_exported(rtg_lib):
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(rtg_lib, n), n


def test_binding_list_matches_header():
    from rti_gb300 import _lib
    assert sorted(_lib.EXPORTS) == sorted(_declared())


def test_abi_version_and_defaults(rtg_lib):
    from rti_gb300 import _lib
    assert rtg_lib.rtg_abi_version() == 1
    c = _lib.default_config()
    assert c.x_bound == _lib.RTG_BOUND_REFLECTIVE and c.y_bound == _lib.RTG_BOUND_REFLECTIVE
    assert c.tnear == float(np.float32(1e-4)) and c.roulette_threshold == 0.1 and c.roulette_weight == 0.3
    assert c.source_exponent == 1.0 and c.box_mode == _lib.RTG_BOX_FROM_GEOMETRY


def test_null_arguments_are_rejected_without_a_device(rtg_lib):
    assert rtg_lib.rtg_create(None, 0) == 1
    assert rtg_lib.rtg_set_config(None, None) == 1
    assert rtg_lib.rtg_trace(None, 10, 0, None) == 1
    assert rtg_lib.rtg_last_error(None) == b"null context"
    assert rtg_lib.rtg_batch_create(None, 0) == 1
    assert rtg_lib.rtg_batch_add(None, None, None, 1, 0, None) == 1
    assert rtg_lib.rtg_autotune(None, 10, 0, None, None) == 1
    assert rtg_lib.rtg_set_launch_config(None, None) == 1


def test_launch_config_default(rtg_lib):
    from rti_gb300 import _lib
    lc = _lib.RtgLaunchConfig()
    rtg_lib.rtg_launch_config_default(C.byref(lc))
    assert lc.as_dict() == {"threads_per_block": 128, "packet": 1, "stack_depth": 0,
                            "scheduling": _lib.RTG_SCHED_MEGAKERNEL, "leaf_tests": _lib.RTG_LEAF_IMMEDIATE,
                            "stack_memory": _lib.RTG_STACK_AUTO}


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "rtg.h"
#define F(T, m) printf(#T "." #m " %zu\n", offsetof(T, m))
int main(void) {
  printf("rtg_config %zu\n", sizeof(rtg_config));
  F(rtg_config, x_bound); F(rtg_config, box_mode); F(rtg_config, box_lo); F(rtg_config, box_hi);
  F(rtg_config, tnear); F(rtg_config, roulette_threshold); F(rtg_config, roulette_weight);
  F(rtg_config, max_segments); F(rtg_config, job);
  printf("rtg_tally %zu\n", sizeof(rtg_tally));
  F(rtg_tally, errors); F(rtg_tally, trace_ms); F(rtg_tally, kernel_ms);
  printf("rtg_device_view %zu\n", sizeof(rtg_device_view));
  F(rtg_device_view, estimates); F(rtg_device_view, n);
  printf("rtg_launch_config %zu\n", sizeof(rtg_launch_config));
  F(rtg_launch_config, packet); F(rtg_launch_config, stack_depth); F(rtg_launch_config, scheduling);
  F(rtg_launch_config, leaf_tests); F(rtg_launch_config, stack_memory);
  printf("rtg_segment %zu\n", sizeof(rtg_segment));
  F(rtg_segment, segment); F(rtg_segment, kind); F(rtg_segment, org); F(rtg_segment, end);
  F(rtg_segment, primitive); F(rtg_segment, weight);
  return 0;
}
"""


def test_struct_layout_matches_ctypes(tmp_path):
    from rti_gb300 import _lib
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.split("\n") if line)
    structs = {"rtg_config": _lib.RtgConfig, "rtg_tally": _lib.RtgTally, "rtg_device_view": _lib.RtgDeviceView,
               "rtg_launch_config": _lib.RtgLaunchConfig, "rtg_segment": _lib.RtgSegment}
    for key, val in out.items():
        if "." in key:
            s, m = key.split(".")
            assert getattr(structs[s], m).offset == int(val), key
        else:
            assert C.sizeof(structs[key]) == int(val), key
    import numpy as np
    assert np.dtype(_lib.SEGMENT_DTYPE).itemsize == C.sizeof(_lib.RtgSegment) == 48


def test_cpp_dropin_header_compiles(tmp_path):
    """include/rti/device.hpp (the rti::device drop-in) compiles with g++ against rtg.h."""
    src = tmp_path / "use.cpp"
    src.write_text('#include "rti/device.hpp"\n'
                   'struct p : rti::particle::i_particle<float> {\n'
                   '  float get_sticking_probability(RTCRay&, RTCHit&, rti::geo::meta_geometry<float>&,\n'
                   '                                 rti::rng::i_rng&, rti::rng::i_rng::i_state&) override { return 0.1f; }\n'
                   '  void init_new() override {}\n};\n'
                   'int main() { rti::device<float, p, rti::reflection::diffuse<float>> d; d.set_number_of_rays(10);'
                   ' d.set_multi_hit_window(5.0f);'
                   ' return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
