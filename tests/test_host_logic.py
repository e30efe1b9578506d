"""Host-side logic that needs no GPU: the C-ABI library and its exports, the parameter-struct layouts, the
Python mirror of the reference containers, bench helpers and the replica timing reduction over 2 gloo ranks."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(mraygb_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    from mray_gb300 import _lib

    L = _lib.load()
    declared = declared_symbols()
    assert len(declared) >= 16
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) == declared


def test_struct_layouts_match_the_c_header(tmp_path):
    """sizeof / offsetof of the POD mirrors as gcc lays out include/mraygb_types.h, against the ctypes mirrors."""
    from mray_gb300.types import (Camera, ErrorReconstructionParameters, GenerationParameters, MomentImageArrays,
                                  ReconstructionParameters, ReferenceParameters, SingleScatteringParameters,
                                  UncertaintyReconstructionParameters)

    src = tmp_path / "layout.c"
    classes = {"mraygb_camera": Camera, "mraygb_generation_params": GenerationParameters,
               "mraygb_reconstruction_params": ReconstructionParameters,
               "mraygb_error_params": ErrorReconstructionParameters,
               "mraygb_uncertainty_params": UncertaintyReconstructionParameters,
               "mraygb_single_scattering_params": SingleScatteringParameters,
               "mraygb_reference_params": ReferenceParameters, "mraygb_moment_image": MomentImageArrays}
    fields = {st: [f[0] for f in cls._fields_] for st, cls in classes.items()}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/mraygb_types.h"', 'int main(){']
    for st, fl in fields.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fl:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.splitlines())
    for st, cls in classes.items():
        assert int(out[st]) == C.sizeof(cls)
        for f in fields[st]:
            assert int(out[f"{st}.{f}"]) == getattr(cls, f).offset, f


def test_defaults_mirror_the_reference():
    from mray_gb300 import GenerationParameters, ReconstructionParameters

    g = GenerationParameters()
    assert (g.step_size, g.error_threshold, g.compact_image, g.prediction_coding, g.quantization_bits,
            g.coding_warp, g.transform_to_bounds) == (1.0, 1.0, 1, 1, 32, 0, 0)
    assert abs(g.bias - 1e-4) < 1e-10 and abs(g.transform_bound_eps - 0.01) < 1e-9
    r = ReconstructionParameters()
    assert abs(r.bias - 1e-6) < 1e-12 and abs(r.early_ray_termination - 0.95) < 1e-7
    assert abs(r.step_size - 0.01) < 1e-9 and abs(r.medium_emission - 0.1) < 1e-8


def test_moment_image_accessors():
    import mray_gb300 as M

    mi = M.MomentImageHost(8, 4, 10, True, True)
    counts = np.tile(np.arange(8), 4)
    mi.index[1:] = np.cumsum(counts)
    mi.is_compact = True
    assert mi.get_num_moments(3, 0) == 3 and mi.get_idx(4, 0) == 6
    mi.bounds[:] = (0, 65535)
    assert mi.get_bounds(1, 1) == (0.0, 1.0)


def test_preintegrate_matches_oracle():
    import mray_gb300 as M
    import oracle as O
    from mray_gb300 import workloads as W

    tf1d = W.transfer_function(3)
    assert np.array_equal(M.preintegrate(tf1d, 0.037).table, O.preintegrate(tf1d, 0.037))


def test_default_quantization_table():
    import mray_gb300 as M

    t = M.default_quantization_table(64, 10)
    assert t[0] == 16 and np.all(t[1:] == 10) and t.size == 64


def test_no_gpu_fails_cleanly():
    """Without a usable device, creating a context reports an error status instead of aborting."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import mray_gb300 as M

    with pytest.raises(M.MrayError):
        M.Context(0)


def test_samples_per_ray_counts_the_march():
    sys.path.insert(0, ROOT)
    import bench
    from mray_gb300 import workloads as W

    wl = W.ml_workload(n=16, width=24, height=16, num_moments=4, seed=2)
    s = bench.samples_per_ray(wl)
    assert s.shape == (16, 24) and s.max() > 0
    # rays through the [-1, 1]^3 box in 1/16 steps: at most sqrt(12) / (1/16) + 1 samples
    assert s.max() <= int(np.sqrt(12) * 16) + 2


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    vals = bench.reduce_max([1.0 + rank, 10.0 - rank], dist, "cpu")
    dist.barrier()
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(" ".join(str(v) for v in vals))
    dist.destroy_process_group()


def test_replica_timing_max_over_two_gloo_ranks(tmp_path):
    import socket

    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert (tmp_path / f"r{r}.txt").read_text().split() == ["2.0", "10.0"]
