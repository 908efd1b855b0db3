"""Builds a host (CPU) emulation of library kernel sources for tests.

The chosen .cu files of vardyn_gb300/csrc are copied into a build folder next
to the emulation header (tests/host_emulation/vd_internal.cuh), every kernel
launch ``name<<<grid, block, smem, stream>>>(args);`` is rewritten into a call
of ``vd_emu::launch``, and g++ compiles them into one shared library. Kernels
of files listed as cooperative (block-stride loops separated by barriers) run
with one-thread blocks; the others run every thread of the grid in turn.
Test infrastructure only: the product library is built by nvcc
(vardyn_gb300/build.py)."""
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "vardyn_gb300", "csrc")


def _rewrite(src, coop):
    out, pos = [], 0
    for m in re.finditer(r"<<<", src):
        if m.start() < pos:
            continue
        line0 = src.rfind("\n", 0, m.start()) + 1
        head = src[line0:m.start()]
        name = head.strip()
        indent = head[:len(head) - len(head.lstrip())]
        end_cfg = src.index(">>>", m.end())
        cfg = src[m.end():end_cfg]
        i = end_cfg + 3
        assert src[i] == "(", src[line0:i + 20]
        depth, j = 0, i
        while True:
            c = src[j]
            if c == "(":
                depth += 1
            elif c == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        args = src[i + 1:j]
        assert src[j + 1] == ";", src[line0:j + 5]
        out.append(src[pos:line0])
        out.append(f"{indent}vd_emu::launch({'true' if coop else 'false'}, [&]() {{ {name}({args}); }}, {cfg});")
        pos = j + 2
    out.append(src[pos:])
    return "".join(out)


def build(outdir, files=("vd_sw.cu", "vd_neumann.cu"), coop=("vd_neumann.cu",)):
    os.makedirs(outdir, exist_ok=True)
    srcs = []
    for f in files:
        with open(os.path.join(CSRC, f)) as fh:
            text = _rewrite(fh.read(), f in coop)
        dst = os.path.join(outdir, f[:-3] + ".cpp")
        with open(dst, "w") as fh:
            fh.write(text)
        srcs.append(dst)
    for f in ("vd_internal.cuh", "emu_runtime.cpp"):
        with open(os.path.join(HERE, f)) as fh, open(os.path.join(outdir, f), "w") as gh:
            gh.write(fh.read())
    srcs.append(os.path.join(outdir, "emu_runtime.cpp"))
    lib = os.path.join(outdir, "libvd_emu.so")
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-w", f"-I{outdir}", f"-I{os.path.join(ROOT, 'include')}",
           "-o", lib] + srcs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host emulation build failed:\n" + r.stderr[-4000:])
    return lib
