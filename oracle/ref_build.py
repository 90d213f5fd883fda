"""Builds oracle/_ref/refcheck: the reference's own shader math, compiled on the CPU, checked
against the oracle's restatement on the same inputs.

TEST INFRASTRUCTURE ONLY. Reads the reference's shader sources where they lie
(/root/reference/Source/Renderer/shaders, or $YAPT_REFERENCE_SHADERS), applies mechanical
edits that make HLSL compile as C++ together with oracle/hlsl_shim.h, and writes the edited
copies and the binary into oracle/_ref/ only (git-ignored; never committed):

  * `out T name` / `inout T name` parameters become `T& name` (arrays: `T (&name)[N]`), and
    the `in` qualifier is dropped;
  * unsuffixed floating literals get an `f` suffix (HLSL literals are float, C++ double), and
    `1.#INF` becomes INFINITY;
  * comments, register bindings, Vulkan binding attributes and loop attributes are dropped;
    unsized resource arrays get a size; a cast of zero `(Type)0` becomes `Type{}` (HLSL casts
    a scalar to a struct member by member);
  * include directives are resolved case-insensitively (the shaders were written on Windows).

The struct SurfaceDefinition (raytracing/hitShadersCommon.hlsl) and the subsurface functions of
raytracing/subsurface.hlsl other than its probe-ray sampler are extracted on their own, so the
ray-tracing resources those files pull in are not needed.

  python oracle/ref_build.py            # build (skips quietly when the shaders are absent)
  python oracle/ref_build.py --run      # build and run the comparison, print its JSON
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SHADERS = os.environ.get("YAPT_REFERENCE_SHADERS", "/root/reference/Source/Renderer/shaders")
OUT = os.path.join(HERE, "_ref")
HLSL_OUT = os.path.join(OUT, "hlsl")
BIN = os.path.join(OUT, "refcheck")

FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
OUT_ARRAY = re.compile(r"\b(?:inout|out)\s+([A-Za-z_]\w*)\s+([A-Za-z_]\w*)\s*\[([^\]]+)\]")
OUT_PARAM = re.compile(r"\b(?:inout|out)\s+([A-Za-z_][\w:]*(?:<[^>]*>)?)\s+([A-Za-z_]\w*)")
IN_PARAM = re.compile(r"([(,]\s*)in\s+(?=[A-Za-z_])")
REGISTER = re.compile(r":\s*register\s*\([^)]*\)")
VK_ATTR = re.compile(r"\[\[vk::[^\]]*\]\]")
LOOP_ATTR = re.compile(r"\[(?:unroll|loop|branch|flatten|fastopt|call|forcecase)(?:\([^)]*\))?\]")
STRUCT_ZERO = re.compile(r"\(\s*([A-Za-z_]\w*)\s*\)\s*0(?:\.0*)?f?(?![\w.])")
LINE_COMMENT = re.compile(r"//[^\n]*")
BLOCK_COMMENT = re.compile(r"/\*.*?\*/", re.S)
UNSIZED = re.compile(r"^(\s*[A-Za-z_][\w<>]*\s+\w+)\s*\[\s*\]\s*;", re.M)
INCLUDE = re.compile(r'^(\s*#\s*include\s*")([^"]+)(")', re.M)


def _suffix_floats(line):
    # leave comments and preprocessor lines other than #define alone
    code, sep, comment = line.partition("//")
    if code.lstrip().startswith("#") and not code.lstrip().startswith("#define"):
        return line
    return FLOAT_LIT.sub(lambda m: m.group(1) + "f", code) + sep + comment


def _resolve(dirpath, rel):
    """Case-insensitive include resolution relative to dirpath (inside the shader tree)."""
    cur = dirpath
    for part in rel.replace("\\", "/").split("/"):
        if part in ("", "."):
            continue
        if part == "..":
            cur = os.path.dirname(cur)
            continue
        names = {n.lower(): n for n in os.listdir(cur)}
        if part.lower() not in names:
            return None
        cur = os.path.join(cur, names[part.lower()])
    return cur


def transform(text, src_path):
    text = BLOCK_COMMENT.sub(lambda m: "\n" * m.group(0).count("\n"), text)
    text = LINE_COMMENT.sub("", text)
    text = text.replace("1.#INF", "INFINITY")
    text = VK_ATTR.sub("", text)
    text = REGISTER.sub("", text)
    text = LOOP_ATTR.sub("", text)
    text = OUT_ARRAY.sub(r"\1 (&\2)[\3]", text)
    text = OUT_PARAM.sub(r"\1& \2", text)
    text = IN_PARAM.sub(r"\1", text)
    text = STRUCT_ZERO.sub(r"\1{}", text)
    text = UNSIZED.sub(r"\1[64];", text)
    text = re.sub(r"\bgroupshared\b", "static", text)
    text = "\n".join(_suffix_floats(ln) for ln in text.split("\n"))

    def inc(m):
        target = _resolve(os.path.dirname(src_path), m.group(2))
        if target is None:
            return m.group(0)
        rel = os.path.relpath(target, os.path.dirname(src_path)).replace(os.sep, "/")
        return m.group(1) + rel + m.group(3)

    return INCLUDE.sub(inc, text)


def extract_struct(text, name):
    m = re.search(r"\bstruct\s+%s\b[^{]*\{" % re.escape(name), text)
    if not m:
        raise RuntimeError("struct %s not found" % name)
    depth, i = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(text[i], 0)
        i += 1
    j = text.index(";", i)
    return text[m.start():j + 1]


def extract_function(text, name):
    """The definition of function `name` (return type through the closing brace)."""
    m = re.search(r"^[ \t]*[A-Za-z_][\w<>]*[ \t]+%s[ \t]*\(" % re.escape(name), text, re.M)
    if not m:
        raise RuntimeError("function %s not found" % name)
    i = text.index("{", m.end())
    depth, j = 1, i + 1
    while depth:
        depth += {"{": 1, "}": -1}.get(text[j], 0)
        j += 1
    return text[m.start():j]


# the subsurface functions compared (subsurface.hlsl); its probe-ray sampler needs the ray-query
# pipeline and stays out
SUBSURFACE_FUNCTIONS = ["getSubsurfaceLayerWeight", "getEnergyLeftForBaseLayer", "getSubsurfaceEntryFactor", "burleyScale",
                        "burleyD", "burleyRMax", "burleyProfileArea", "burleySampleRadius", "evaluateSubsurfaceRd",
                        "getSubsurfaceProbeFrame", "getSubsurfaceProbeAxisProbability", "pdfSubsurfaceExit",
                        "sampleSubsurfaceExitLobe", "evaluateSubsurfaceExitLobe"]


def convert_tree():
    for dirpath, _, files in os.walk(SHADERS):
        for f in files:
            if not f.endswith((".hlsl", ".h")):
                continue
            src = os.path.join(dirpath, f)
            dst = os.path.join(HLSL_OUT, os.path.relpath(src, SHADERS))
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(src, encoding="utf-8", errors="replace") as fh:
                text = fh.read()
            with open(dst, "w") as fh:
                fh.write(transform(text, src))
    hsc = os.path.join(SHADERS, "raytracing", "hitShadersCommon.hlsl")
    with open(hsc, encoding="utf-8", errors="replace") as fh:
        piece = extract_struct(fh.read(), "SurfaceDefinition")
    with open(os.path.join(HLSL_OUT, "SurfaceDefinition.inc"), "w") as fh:
        fh.write(transform(piece, hsc) + "\n")
    sss = os.path.join(SHADERS, "raytracing", "subsurface.hlsl")
    with open(sss, encoding="utf-8", errors="replace") as fh:
        text = fh.read()
    defines = "\n".join(ln for ln in text.split("\n") if ln.startswith("#define SUBSURFACE_"))
    parts = [defines] + [extract_function(text, f) for f in SUBSURFACE_FUNCTIONS]
    with open(os.path.join(HLSL_OUT, "subsurface_math.inc"), "w") as fh:
        fh.write(transform("\n\n".join(parts), sss) + "\n")


def build():
    if not os.path.isdir(SHADERS):
        print("reference shaders not present (%s): oracle/_ref not built" % SHADERS)
        return False
    os.makedirs(OUT, exist_ok=True)
    convert_tree()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    flags = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-w", "-I" + HERE,
             "-I" + os.path.join(cuda, "include")]
    srcs = [os.path.join(HERE, "refcheck", s) for s in ("hlsl_side.cpp", "hlsl_side_kulla.cpp", "oracle_side.cpp", "main.cpp")]
    srcs.append(os.path.join(ROOT, "yapt_gb300", "csrc", "yg_tables.cpp"))
    objs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        r = subprocess.run(["g++"] + flags + ["-c", s, "-o", o], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout)
            raise RuntimeError("compiling %s failed" % s)
        objs.append(o)
    r = subprocess.run(["g++", "-pthread", "-o", BIN] + objs, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("linking refcheck failed")
    return True


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--run", action="store_true")
    ap.add_argument("--samples", type=int, default=20000)
    a = ap.parse_args()
    if build() and a.run:
        data_dir = os.path.join(ROOT, "yapt_gb300", "data")
        r = subprocess.run([BIN, data_dir, str(a.samples)], stdout=subprocess.PIPE, text=True)
        print(r.stdout)
        sys.exit(r.returncode)


if __name__ == "__main__":
    main()
