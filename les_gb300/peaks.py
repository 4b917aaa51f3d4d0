"""Measures the FP64 / FP32 FMA rates and copy bandwidth of the local GPU
with the stand-alone probe csrc/peak_probe.cu.

  python -m les_gb300.peaks          (prints the probe's report)
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def run():
    out = os.path.join(HERE, "_build", "peak_probe")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    src = os.path.join(HERE, "csrc", "peak_probe.cu")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", out, src], check=True)
    r = subprocess.run([out], capture_output=True, text=True, check=True)
    txt = r.stdout
    fp64 = [float(x) for x in re.findall(r"fp64 fma: .* ([0-9.]+) TFLOP/s", txt)]
    fp32 = [float(x) for x in re.findall(r"fp32 fma: .* ([0-9.]+) TFLOP/s", txt)]
    cp = [float(x) for x in re.findall(r"copy: .* ([0-9.]+) GB/s", txt)]
    return {"fp64_tflops": max(fp64) if fp64 else None, "fp32_tflops": max(fp32) if fp32 else None,
            "copy_gbs": max(cp) if cp else None, "raw": txt}


if __name__ == "__main__":
    d = run()
    sys.stdout.write(d["raw"])
    print({k: v for k, v in d.items() if k != "raw"})
