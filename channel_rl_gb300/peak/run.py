"""Measure the FP64 (DFMA/DADD), DDIV, DSQRT and FP32 FFMA issue rates of
this GPU and write profiles/fp64_peak.json.

The channel step is FP64-bound on GB300, so its roofline uses the measured
DFMA rate (one DFMA = 2 flops).

    python -m channel_rl_gb300.peak.run
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
        exe = os.path.join(d, "fp64_peak")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                        os.path.join(HERE, "fp64_peak.cu")], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    print(out)
    res = {"raw": out.strip().splitlines()}
    for name, key in (("DFMA", "dfma"), ("DADD", "dadd"), ("DDIV", "ddiv"), ("DSQRT", "dsqrt"), ("FFMA", "ffma")):
        m = re.search(rf"^{name}: [0-9.]+ ms, ([0-9.]+) G", out, re.M)
        if m:
            res[key + "_gops"] = float(m.group(1))
    if "dfma_gops" in res:
        res["dfma_gflops"] = 2.0 * res["dfma_gops"]
    res["how"] = ("8 independent dependency chains per thread, 152x8 blocks x 256 threads, "
                  "CUDA events, third repetition; thread-instructions per second")
    os.makedirs(os.path.join(ROOT, "profiles"), exist_ok=True)
    with open(os.path.join(ROOT, "profiles", "fp64_peak.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
