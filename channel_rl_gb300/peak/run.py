"""Measure the FP64 (DFMA, DADD, a DFMA/DADD/DMUL mix), DDIV, DSQRT and FP32
FFMA issue rates of this GPU and write profiles/fp64_peak.json.

The channel step is FP64-bound on GB300, so its roofline uses the measured
FP64 issue rate: the largest rate over the probes and swept chain counts
(`fp64_peak_gops`, a DFMA loop on register operands; one DFMA = 2 flops).

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


def summarise(out):
    """The probe's output as the fp64_peak.json record."""
    res = {"raw": out.strip().splitlines()}
    m = re.search(r"^BEST dfma ([0-9.]+) dadd ([0-9.]+) mixed ([0-9.]+) ddiv ([0-9.]+) dsqrt ([0-9.]+) ffma ([0-9.]+)"
                  r" reg ([0-9.]+)", out, re.M)
    if m:
        for key, v in zip(("dfma", "dadd", "mixed", "ddiv", "dsqrt", "ffma", "reg_operands"), m.groups()):
            res[key + "_gops"] = float(v)
        res["fp64_peak_gops"] = max(res["dfma_gops"], res["dadd_gops"], res["mixed_gops"], res["reg_operands_gops"])
        res["dfma_gflops"] = 2.0 * res["fp64_peak_gops"]
    # DFMA reading three different registers each (no operand reuse), the
    # form of the stencil kernels' FMAs: the practical rate for such code
    distinct = [float(x) for x in re.findall(r"^DFMA 3 distinct regs x\d+ chains: [0-9.]+ ms, ([0-9.]+) Gop/s", out, re.M)]
    if distinct:
        res["dfma_distinct_operands_gops"] = max(distinct)
    res["how"] = ("8, 16 and 32 independent dependency chains per thread (loop unrolled 4x), 152x8 blocks x 256 "
                  "threads, CUDA events, third repetition, best of the sweep; thread-instructions per second; "
                  "operands from the constant bank, and from registers in the reg_operands probes")
    return res


def main():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "fp64_peak")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                        os.path.join(HERE, "fp64_peak.cu")], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    print(out)
    res = summarise(out)
    os.makedirs(os.path.join(ROOT, "profiles"), exist_ok=True)
    with open(os.path.join(ROOT, "profiles", "fp64_peak.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
