"""Host-side checks of the serving layer (no GPU): the arena sub-allocator, the ctypes mirrors of
the C structs, and the error a server reports on a machine without a GPU."""
import ctypes
import os
import subprocess

import pytest

from pnepma_gb300 import capi
from pnepma_gb300.material_model import PnMaterialDesc, PnSlices
from pnepma_gb300.problem import PnDesc, PnSizes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile_and_run(tmp_path, src, lang, flags):
    exe = str(tmp_path / "a.out")
    compiler = "g++" if lang == "c++" else "gcc"
    r = subprocess.run([compiler] + flags + [src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_arena_invariants(tmp_path):
    out = _compile_and_run(tmp_path, os.path.join(ROOT, "tests", "native", "arena_check.cpp"), "c++",
                           ["-std=c++17", "-O2", "-I", os.path.join(ROOT, "pnepma_gb300", "csrc")])
    assert out.strip() == "ok"


STRUCTS = {
    "pn_desc": PnDesc, "pn_sizes": PnSizes, "pn_batch_options": capi.PnBatchOptions,
    "pn_batch_info": capi.PnBatchInfo, "pn_handle_info": capi.PnHandleInfo,
    "pn_server_options": capi.PnServerOptions, "pn_request": capi.PnRequest,
    "pn_ticket_info": capi.PnTicketInfo, "pn_server_info": capi.PnServerInfo,
    "pn_slices": PnSlices, "pn_material_desc": PnMaterialDesc,
}


def test_ctypes_structs_match_the_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pnepma.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append(f'  printf("{name} %zu\\n", sizeof({name}));')
        for f in cls._fields_:
            lines.append(f'  printf("{name}.{f[0]} %zu\\n", offsetof({name}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    out = _compile_and_run(tmp_path, str(src), "c", ["-std=c11", "-I", os.path.join(ROOT, "include")])
    got = dict(l.rsplit(" ", 1) for l in out.strip().splitlines())
    for name, cls in STRUCTS.items():
        assert int(got[name]) == ctypes.sizeof(cls), name
        for f in cls._fields_:
            assert int(got[f"{name}.{f[0]}"]) == getattr(cls, f[0]).offset, f"{name}.{f[0]}"


def test_server_without_a_device_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.PnError) as e:
        capi.Server(memory_budget=1 << 20)
    assert e.value.code == -9
