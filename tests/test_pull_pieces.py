"""Host logic of the gathered copy (hs_internal.h, pull_add): a copy is cut into
contiguous pieces of at most PULL_CHUNK_BYTES that cover it exactly, in order.
Compiled with g++ against the CUDA runtime headers; CPU only."""

import os
import shutil
import subprocess
from pathlib import Path

import pytest

import _cpp
from conftest import ROOT

PROGRAM = r"""
#include <cstdio>
#include "hs_internal.h"
int main()
{
    const size_t sizes[] = {0, 1, 15, 16, hs::PULL_CHUNK_BYTES - 1, hs::PULL_CHUNK_BYTES, hs::PULL_CHUNK_BYTES + 1,
                            3 * hs::PULL_CHUNK_BYTES - 5, 10 * hs::PULL_CHUNK_BYTES};
    static unsigned char src[11 << 18], dst[11 << 18];
    std::printf("chunk %zu\n", hs::PULL_CHUNK_BYTES);
    for (size_t b : sizes) {
        std::vector<hs::PullChunk> list;
        hs::pull_add(list, dst + 3, src + 1, b);  // odd offsets: the pieces keep them
        std::printf("copy %zu %zu\n", b, list.size());
        for (const hs::PullChunk &c : list)
            std::printf("%td %td %llu\n", c.src - (src + 1), c.dst - (dst + 3), (unsigned long long)c.bytes);
    }
    return 0;
}
"""


def cuda_include():
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    cands = [Path(home) / "include"] if home else []
    nvcc = shutil.which("nvcc")
    if nvcc:
        cands.append(Path(nvcc).resolve().parent.parent / "include")
    cands.append(Path("/usr/local/cuda/include"))
    for c in cands:
        if (c / "cuda_runtime.h").exists():
            return c
    return None


def test_copy_pieces_cover_each_copy(tmp_path):
    inc = cuda_include()
    if inc is None:
        pytest.skip("CUDA runtime headers not found")
    src = tmp_path / "pieces.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "pieces"
    r = subprocess.run([_cpp.gxx(), "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{inc}",
                        f"-I{ROOT / 'helioselene_gb300' / 'csrc'}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    chunk = int(lines[0].split()[1])
    assert chunk == 256 << 10
    i, copies = 1, 0
    while i < len(lines) and lines[i].startswith("copy"):
        _, b, k = lines[i].split()
        b, k = int(b), int(k)
        pieces = [tuple(int(x) for x in lines[i + 1 + j].split()) for j in range(k)]
        assert k == -(-b // chunk)
        pos = 0
        for s_off, d_off, size in pieces:
            assert s_off == d_off == pos and 0 < size <= chunk
            pos += size
        assert pos == b
        i += 1 + k
        copies += 1
    assert copies == 9
