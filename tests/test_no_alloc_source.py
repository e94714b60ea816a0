"""The allocation-free spectral transform names no allocation call: the
source of axi_fd_transform_static_f64 and of the helpers it uses (everything
from its section marker to the end of pyaxisymflow_gb300/csrc/gemm_f64.cu)
contains neither cudaMalloc nor cudaFree (nor their driver-API forms)."""
import os
import re

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_static_transform_source_has_no_allocation_call():
    path = os.path.join(HERE, "pyaxisymflow_gb300", "csrc", "gemm_f64.cu")
    src = open(path).read()
    start = src.index("// Allocation-free variant of axi_fd_transform_f64.")
    tail = src[start:]
    assert "axi_fd_transform_static_f64" in tail
    code = re.sub(r"//[^\n]*", "", tail)
    for name in ("cudaMalloc", "cudaFree", "cuMemAlloc", "cuMemFree", "cudaMallocAsync"):
        assert name not in code, name
