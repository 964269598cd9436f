"""Builds the reference's own DTS / HFBS sources for the CPU -- TEST
INFRASTRUCTURE ONLY (the golden vectors under tests/golden/ref_* come from
it; no product code loads it).

The reference (akashbapat/domain_transform_solver, src/) is CUDA C++ whose
kernels, apart from its CUB row scan, are independent per thread.  This
recipe compiles those sources with g++ against stand-ins for the CUDA
runtime, libcua and CUB (oracle/refemu/include) and runs each kernel launch
on the host (refemu.h).  The only change made to the reference's text is
mechanical and is written to oracle/_ref/gen/, never into the repository:
each launch `K<<<grid, block>>>(args)` becomes
`::refemu::launch(dim3(grid), dim3(block), [&]() { K(args); })`
(`launch_coop` for kernels that call __syncthreads()), and the rewritten
files are deleted once the library is built.  Files without a launch are
compiled where they lie.

Usage: python oracle/refemu/build_ref.py [--src DIR]   (default: the
reference checkout's src/ directory, or $DTS_REFERENCE_SRC).
Output: oracle/_ref/libdtsref.so
"""
from __future__ import annotations

import argparse
import os
import platform
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
DEFAULT_SRC = Path(os.environ.get("DTS_REFERENCE_SRC", "/root/reference/src"))

# The translation units of the path (the CLIs, the OpenCV-based helpers and
# the dataset loaders are not part of it).
UNITS = ["domain_transform_filter.cu", "domain_transform_solver.cu", "hfbs.cu",
         "domain_transform_stereo.cu", "error_types.cpp"]


def _match_back(text: str, end: int, open_c: str, close_c: str) -> int:
    """Index of the `open_c` matching the `close_c` at text[end]."""
    depth = 0
    for i in range(end, -1, -1):
        if text[i] == close_c:
            depth += 1
        elif text[i] == open_c:
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced " + open_c + close_c)


def _match_fwd(text: str, start: int, open_c: str, close_c: str) -> int:
    """Index just past the `close_c` matching the `open_c` at text[start]."""
    depth = 0
    for i in range(start, len(text)):
        if text[i] == open_c:
            depth += 1
        elif text[i] == close_c:
            depth -= 1
            if depth == 0:
                return i + 1
    raise ValueError("unbalanced " + open_c + close_c)


def _split_top(s: str) -> list[str]:
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def coop_kernels(texts: list[str]) -> set[str]:
    """Names of __global__ functions whose body calls __syncthreads()."""
    names = set()
    for text in texts:
        for m in re.finditer(r"__global__[^;{]*?\b(\w+)\s*\(", text):
            body_start = text.find("{", m.end())
            if body_start < 0:
                continue
            body_end = _match_fwd(text, body_start, "{", "}")
            if "__syncthreads" in text[body_start:body_end]:
                names.add(m.group(1))
    return names


def rewrite_launches(text: str, coop: set[str]) -> tuple[str, int]:
    n = 0
    while True:
        k = text.find("<<<")
        if k < 0:
            return text, n
        # kernel expression: an identifier, possibly with template arguments
        j = k - 1
        while text[j].isspace():
            j -= 1
        if text[j] == ">":
            j = _match_back(text, j, "<", ">") - 1
            while text[j].isspace():
                j -= 1
        e = j + 1
        while j >= 0 and (text[j].isalnum() or text[j] in "_:"):
            j -= 1
        kstart = j + 1
        name = text[kstart:e].split("::")[-1]
        kernel = text[kstart:k].strip()
        # launch configuration
        depth, c = 0, k + 3
        while True:
            if text[c] in "([{":
                depth += 1
            elif text[c] in ")]}":
                depth -= 1
            elif depth == 0 and text.startswith(">>>", c):
                break
            c += 1
        cfg = _split_top(text[k + 3:c])
        a = c + 3
        while text[a].isspace():
            a += 1
        if text[a] != "(":
            raise ValueError(f"launch of {kernel} without an argument list")
        a_end = _match_fwd(text, a, "(", ")")
        args = text[a + 1:a_end - 1]
        fn = "launch_coop" if name in coop else "launch"
        repl = (f"::refemu::{fn}(dim3({cfg[0]}), dim3({cfg[1]}), [&]() {{ "
                f"{kernel}({args}); }})")
        text = text[:kstart] + repl + text[a_end:]
        n += 1


def build(src: Path = DEFAULT_SRC, force: bool = False) -> Path:
    lib = OUT / "libdtsref.so"
    driver = HERE / "ref_driver.cpp"
    deps = [driver, Path(__file__)] + sorted((HERE / "include").glob("*"))
    if (not force and lib.exists()
            and lib.stat().st_mtime >= max(p.stat().st_mtime for p in deps)):
        return lib
    if not src.is_dir():
        raise FileNotFoundError(f"reference sources not found at {src}")
    gen = OUT / "gen"
    gen.mkdir(parents=True, exist_ok=True)
    files = sorted(p for p in src.iterdir()
                   if p.suffix in (".cu", ".cuh", ".h") and not p.name.startswith("benchmark"))
    texts = {p.name: p.read_text() for p in files}
    coop = coop_kernels(list(texts.values()))
    for name, text in texts.items():
        if "<<<" in text:
            new, n = rewrite_launches(text, coop)
            (gen / name).write_text(new)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=fast",
           "-w", f"-I{gen}", f"-I{src}", f"-I{HERE / 'include'}"]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd.append("-mfma")  # nvcc contracts a*b+c to fma; so does g++ with this
    cmd += [str(driver), "-o", str(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    for p in gen.iterdir():
        p.unlink()
    gen.rmdir()
    if r.returncode != 0:
        raise RuntimeError("reference CPU build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-6000:])
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", type=Path, default=DEFAULT_SRC)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.src, a.force))
    sys.exit(0)
