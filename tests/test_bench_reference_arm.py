"""bench.py --impl reference on the host cores: one JSON line on rank 0 carrying the
metric, the CPU baseline that produced it and an end-to-end figure with no
host-device traffic (the reference runs on the host)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "gemm_8x8192x8_u1u1", "--steps", "3", "--warmup", "1"],
                         env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["unit"] == "GOPS" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["config"]["workload"] == "gemm_8x8192x8_u1u1"
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "GOPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert cb["one_core"]["cores"] == 1 and cb["one_core"]["value"] > 0
    # the same config dict as the GPU arm's line (bench_config), so the two lines compare as one workload
    sys.path.insert(0, ROOT)
    import bench
    M, K, N = 8, 8192, 8
    assert line["config"] == bench.bench_config(bench.workload_desc("gemm_8x8192x8_u1u1"), M, K, N, 1, 1)


def test_resident_contexts_exceed_twice_the_l2():
    sys.path.insert(0, ROOT)
    import bench
    for (M, K, N, wA, wB) in [(2048, 4096, 2048, 3, 2), (256, 9216, 4096, 1, 4), (8, 8192, 8, 1, 1),
                              (4096, 2048, 2048, 2, 1)]:
        P = bench.resident_contexts(M, K, N, wA, wB)
        per = (M + N) * K * (1 + max(wA, wB) / 8.0) + 4.0 * M * N
        assert 2 <= P <= 16
        assert P == 16 or P * per >= 2 * bench.L2_BYTES
