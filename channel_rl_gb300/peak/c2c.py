"""Measure host<->device bandwidth (pinned buffers, copy engines and direct
kernel access) and write profiles/c2c_bandwidth.json: the floor of the
per-step transfers in bench.py's end-to-end line.

    python -m channel_rl_gb300.peak.c2c
"""
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "c2c_peak")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                        os.path.join(HERE, "c2c_peak.cu")], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    print(out)
    res = {"raw": out.strip().splitlines()}
    for key, pat in (("memcpy_h2d_gbs", r"^memcpy H2D ([0-9.]+)"), ("memcpy_d2h_gbs", r"^memcpy D2H ([0-9.]+)"),
                     ("kernel_read_host_gbs", r"^kernel read host x8 ([0-9.]+)"),
                     ("kernel_write_host_gbs", r"^kernel write host x8 ([0-9.]+)")):
        m = re.search(pat, out, re.M)
        if m:
            res[key] = float(m.group(1))
    res["how"] = "118 MB pinned buffers (cudaMallocHost), CUDA events, third repetition"
    os.makedirs(os.path.join(ROOT, "profiles"), exist_ok=True)
    with open(os.path.join(ROOT, "profiles", "c2c_bandwidth.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
