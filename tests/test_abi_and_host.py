"""C ABI surface, record layouts, reciprocal accuracy, and the multi-rank
reduction of the benchmark (gloo, two CPU processes)."""
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

import pgs
import pgs_oracle

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "pgs.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(pgs_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_function():
    lib = pgs.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    # The Python wrapper binds every declared entry point except the
    # allocation-free copy, which is meant for native callers.
    assert set(pgs.EXPORTED_SYMBOLS) == set(names) - {"pgs_vram_local_copy_noalloc"}


def test_record_layouts_match_reference_sizes(tmp_path):
    # VertexPosition 16 B, VertexAttribute 24 B, PrimitiveAttribute 32 B, StateVector 16 B
    # (gs/shaders/data_structures.h:55-80,139-144).
    src = tmp_path / "sizes.c"
    src.write_text('#include "pgs.h"\n#include <stdio.h>\nint main(void){printf("%zu %zu %zu %zu %zu\\n",'
                   'sizeof(pgs_vertex_position),sizeof(pgs_vertex_attribute),sizeof(pgs_primitive_attribute),'
                   'sizeof(pgs_state_vector),sizeof(pgs_texture_desc));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)])
    sizes = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    assert sizes == [16, 24, 32, 16, 104]


def test_cuda_backend_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(pgs.PGSError) as e:
        pgs.CudaBackend(0)
    assert e.value.status in (pgs.STATUS_CODES["PGS_ERROR_NO_DEVICE"], pgs.STATUS_CODES["PGS_ERROR_CUDA"])


def test_rcp_fixed_accuracy():
    # rcp_fixed claims ~24 bits (gs/shaders/math_utils.h:24-26).
    lib = pgs_oracle.load_oracle()
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.integers(1, 1 << 32, 4000, dtype=np.uint64), 1 << np.arange(32, dtype=np.uint64),
                           np.array([3, 5, 7, 255, 65535, 0xFFFFFFFF], dtype=np.uint64)])
    for b in vals:
        r = lib.pgs_oracle_rcp_fixed(int(b))
        assert abs(r * float(b) - 1.0) < 2.0 ** -22, (int(b), r)


def test_rcp_float_accuracy():
    lib = pgs_oracle.load_oracle()
    rng = np.random.default_rng(4)
    for v in np.concatenate([rng.uniform(0.25, 4.0, 2000), rng.uniform(1e-3, 1e3, 2000)]).astype(np.float32):
        r = lib.pgs_oracle_rcp_float(float(v))
        assert abs(r * float(v) - 1.0) < 2.0 ** -21
    assert lib.pgs_oracle_rcp_float(0.0) == float("inf")


WORKER = r"""
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="tcp://127.0.0.1:{port}", rank=int(sys.argv[1]), world_size=2)
mine = 10.0 + 5.0 * int(sys.argv[1])
m = bench.max_over_ranks(mine, dist)
fps = bench.replica_throughput(20, 2, m)
print(m, fps)
dist.barrier()
dist.destroy_process_group()
"""


def test_two_rank_replica_timing_reduction():
    """Each rank renders its own replica; the job time is the slowest rank's and
    throughput counts every rank's frames (bench.py --gpus N)."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    code = WORKER.format(root=str(ROOT), port=port)
    with tempfile.NamedTemporaryFile("w", suffix=".py", delete=False) as f:
        f.write(code)
        path = f.name
    try:
        procs = [subprocess.Popen([sys.executable, path, str(r)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                  text=True) for r in range(2)]
        outs = [p.communicate(timeout=120) for p in procs]
    finally:
        os.unlink(path)
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
        m, fps = (float(v) for v in out.split())
        assert m == 15.0
        assert abs(fps - 2 * 20 / 0.015) < 1e-6
