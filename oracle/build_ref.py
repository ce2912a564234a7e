"""Build the CPU parity checkers (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle/am_oracle.c`` into
  ``oracle/_build/libamoracle.so``.
* ``build_ref()`` rewrites the reference's own backend sources (read from the
  reference checkout when it is present) into ``oracle/_ref/gen/`` and
  compiles them with ``oracle/refshim/`` into ``oracle/_ref/libamref.so``: the
  reference's marching loop running on the host cores through OpenMP.  The
  rewrite is mechanical (see ``_rewrite``); the generated sources are
  git-ignored and only ever live under ``oracle/_ref/``.  Where the reference
  checkout is absent (the GPU machine) but ``oracle/_ref/gen/`` travelled with
  the working tree, it compiles from there.

Both builds use ``-ffp-contract=off`` so an x86 and an Arm build round the
same way.
"""
from __future__ import annotations

import glob
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("AM_REFERENCE_ROOT", "/root/reference")
GEN = os.path.join(HERE, "_ref", "gen")
REF_SO = os.path.join(HERE, "_ref", "libamref.so")
ORACLE_SO = os.path.join(HERE, "_build", "libamoracle.so")

_SOURCES = [
    "inc/utilities.h", "inc/macro.h", "inc/facedata.h", "inc/hash.h", "inc/vecmat.h", "inc/mlp.h",
    "inc/states.h", "inc/kernel.h", "inc/polymesh.h", "inc/process.h", "inc/var.h",
    "src/kernel.cu", "src/states.cu", "src/cuam_kernel.cu",
]

_LAUNCH = re.compile(
    r"(?P<name>[A-Za-z_]\w*(?:\s*<[^<>;()]*>)?)\s*<<<\s*(?P<g>[^,<>]+?)\s*,\s*(?P<t>[^<>]+?)\s*>>>\s*"
    r"\((?P<args>.*?)\)\s*;",
    re.DOTALL,
)

_SORT_OLD = re.compile(
    r"auto first = thrust::make_zip_iterator\(.*?thrust::less<int>\(\)\);",
    re.DOTALL,
)


def _cccl_include() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cands = [os.path.join(cuda, "include", "cccl")] + sorted(glob.glob(os.path.join(cuda, "targets", "*", "include", "cccl")))
    for c in cands:
        if os.path.isdir(os.path.join(c, "thrust")):
            return c
    raise RuntimeError("CCCL (thrust) headers not found under %s" % cuda)


def _rewrite(name: str, text: str) -> str:
    """Mechanical host rewrite of one reference source file."""
    for inc in ("<cuda.h>", "<cuda_runtime.h>", "<cublas_v2.h>", "<torch/extension.h>"):
        text = text.replace("#include %s" % inc, '#include "am_ref_shim.h"')
    # kernel<<<grid, block>>>(args);  ->  amref_launch(grid, block, [&]{ kernel(args); });
    text = _LAUNCH.sub(lambda m: "amref_launch((%s), (%s), [&]() { %s(%s); });" % (
        m.group("g"), m.group("t"), m.group("name"), m.group("args")), text)
    if name.endswith("hash.h"):
        # take try_insert's atomicCAS path: the loop runs multi-threaded here
        text = text.replace("#ifndef __CUDA_ARCH__ // CPU", "#if 0 // CPU")
    if name.endswith("macro.h"):
        # silence the per-region "we cannot find solution" kernel printf
        text = text.replace("#define _ENABLE_KERNEL_PRINTF", "// #define _ENABLE_KERNEL_PRINTF")
    if name.endswith("process.h"):
        text, n = _SORT_OLD.subn("amref_sort_segments(value, segments, key_vec, one_batch_len, batch_num);", text)
        assert n == 1, "sortDistance not found"
    if name.endswith("cuam_kernel.cu"):
        # record before inferAndAppend: push_back reuses the popped facedata slots
        old = "inferAndAppend(states_buffer, batch_size, var);"
        assert old in text
        text = text.replace(old, "amref_record(var, states_buffer, faces_buffer, batch_size);\n        " + old)
        old = "var.polymesh.append_verts(var.vertices_buffer, batch_size);"
        assert old in text
        text = text.replace(old, old + "\n        amref_after_batch(var);")
    assert "<<<" not in re.sub(r"//[^\n]*", "", text), "unconverted launch in %s" % name
    return text


def generate(ref_root: str = REF_ROOT) -> bool:
    backend = os.path.join(ref_root, "backend")
    if not os.path.isdir(backend):
        return False
    os.makedirs(GEN, exist_ok=True)
    for rel in _SOURCES:
        with open(os.path.join(backend, rel)) as f:
            text = f.read()
        out = os.path.join(GEN, os.path.basename(rel))
        new = _rewrite(rel, text)
        if os.path.exists(out):
            with open(out) as f:
                if f.read() == new:
                    continue
        with open(out, "w") as f:
            f.write(new)
    return True


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout[-6000:]))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "am_oracle.c")
    deps = [src, os.path.join(HERE, "am_oracle.h"), os.path.join(HERE, "am_oracle_impl.h")]
    if force or _stale(ORACLE_SO, deps):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        tmp = ORACLE_SO + ".tmp"
        _run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", src, "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force: bool = False) -> str | None:
    """Returns the path of libamref.so, or None when neither the reference
    checkout nor previously generated sources are available."""
    generate()
    if not os.path.exists(os.path.join(GEN, "cuam_kernel.cu")):
        return None
    harness = os.path.join(HERE, "refshim", "am_ref_harness.cpp")
    deps = [harness, os.path.join(HERE, "refshim", "am_ref_shim.h")] + glob.glob(os.path.join(GEN, "*"))
    if force or _stale(REF_SO, deps):
        tmp = REF_SO + ".tmp"
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w", "-fpermissive",
              "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP",
              "-I", os.path.join(HERE, "refshim"), "-I", GEN, "-I", _cccl_include(),
              harness, "-o", tmp])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
