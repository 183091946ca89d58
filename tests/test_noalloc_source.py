"""The allocation-free entry point's source names no allocating call (CPU check).

msod_noalloc.cu serves callers that cannot let the library allocate device memory; its code
(comments and string literals aside) must call no cudaMalloc / cudaFree family routine, no host
allocator and none of the library's allocating helpers.
"""
import os
import re

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "minisod2d_gb300", "csrc",
                   "msod_noalloc.cu")

FORBIDDEN = ["cudaMalloc", "cudaFree", "cudaMallocAsync", "cudaFreeAsync", "cudaMallocManaged", "cudaMallocHost",
             "cudaHostAlloc", "cuMemAlloc", "cuMemCreate", "device_flags", "device_tables", "malloc", "calloc",
             "realloc", "new ", "torch"]


def code_only(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    return re.sub(r'"(?:\\.|[^"\\])*"', '""', text)


def test_noalloc_source_names_no_allocating_call():
    code = code_only(open(SRC).read())
    for name in FORBIDDEN:
        pat = r"\b" + re.escape(name.strip()) + (r"\s" if name.endswith(" ") else r"\b")
        assert not re.search(pat, code), name
    assert "cudaGetSymbolAddress" in code
    assert re.search(r"static __device__ __align__\(256\) int g_noalloc_status\[", code)
