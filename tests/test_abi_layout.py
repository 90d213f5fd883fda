"""The ctypes mirrors of the C ABI's structs have the header's layout.

A C program compiled against include/yapt_gpu.h prints sizeof and offsetof of every field the
Python layer declares; each must equal what ctypes computes, so a field added to one side
alone (or reordered) fails here instead of corrupting a call on the GPU."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

from yapt_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "yg_material": N.Material,
    "yg_mesh_desc": N.MeshDesc,
    "yg_instance": N.Instance,
    "yg_camera": N.Camera,
    "yg_punctual_light": N.PunctualLight,
    "yg_tonemap_params": N.TonemapParams,
    "yg_atrous_params": N.AtrousParams,
    "yg_render_params": N.RenderParams,
    "yg_sample_record": N.SampleRecord,
    "yg_kernel_profile": N.KernelProfile,
    "yg_server_options": N.ServerOptions,
    "yg_request": N.Request,
    "yg_request_info": N.RequestInfo,
    "yg_server_stats": N.ServerStats,
    "yg_sched_item": N.SchedItem,
    "yg_nn_tensor": N.NNTensor,
}


def c_layout(tmp):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "yapt_gpu.h"', "int main(void) {"]
    for cname, cls in MIRRORS.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["return 0;", "}"]
    src = os.path.join(tmp, "layout.c")
    exe = os.path.join(tmp, "layout")
    with open(src, "w") as f:
        f.write("\n".join(lines) + "\n")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        struct, field, value = line.split()
        table[(struct, field)] = int(value)
    return table


def test_ctypes_structs_match_the_header():
    with tempfile.TemporaryDirectory() as tmp:
        table = c_layout(tmp)
    mismatches = []
    for cname, cls in MIRRORS.items():
        if table[(cname, "sizeof")] != ctypes.sizeof(cls):
            mismatches.append("%s: sizeof C %d, ctypes %d" % (cname, table[(cname, "sizeof")], ctypes.sizeof(cls)))
        for field, _ in cls._fields_:
            off = getattr(cls, field).offset
            if table[(cname, field)] != off:
                mismatches.append("%s.%s: offset C %d, ctypes %d" % (cname, field, table[(cname, field)], off))
    assert not mismatches, mismatches


def test_header_compiles_cleanly_as_c_and_cpp():
    """A host in either language includes the header with every warning on and nothing else."""
    with tempfile.TemporaryDirectory() as tmp:
        for lang, compiler, std in (("c", "gcc", "-std=c11"), ("cpp", "g++", "-std=c++17")):
            cc = shutil.which(compiler)
            if cc is None:
                pytest.skip("no %s compiler" % compiler)
            src = os.path.join(tmp, "inc." + lang)
            with open(src, "w") as f:
                f.write('#include "yapt_gpu.h"\nint main(void) { return yg_version() > 0 ? 0 : 1; }\n')
            subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                            "-c", src, "-o", os.path.join(tmp, "inc_" + lang + ".o")], check=True)
