"""Regenerates default.tunecache, the launch-shape table the library ships: shapes are taken from
it without timing (after a GBC_TUNE_CACHE file, before autotuning), so that separate processes on
a GB300 run the same kernel shapes and give bitwise-identical results on the workloads it covers.
Run on a GB300, from the repository root:

    python chroma_gb300/tune/make_table.py

It runs bench.py's workloads (one timed step, no CPU legs) and the smoke test with autotuning on,
GBC_TUNE_DEFAULTS=0 and GBC_TUNE_CACHE pointing at a scratch file, then installs that file's
entries (one line per key: device, compute capability, lattice, precision, reconstruction,
epilogue, isign, reduction, right-hand sides, shape-table hash -> shape) next to this script."""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    with tempfile.TemporaryDirectory() as tmp:
        cache = os.path.join(tmp, "tune.cache")
        env = dict(os.environ, GBC_TUNE_CACHE=cache, GBC_TUNE_DEFAULTS="0")
        env.pop("GBC_SHAPE", None)
        env.pop("GBC_AUTOTUNE", None)
        runs = [[sys.executable, "bench.py", "--steps", "1", "--warmup", "1", "--no-cpu-baseline", "--no-oracle-check"],
                [sys.executable, "-c", "import __graft_entry__ as g; g.smoke()"]]
        for cmd in runs:
            subprocess.run(cmd, cwd=ROOT, env=env, check=True, stdout=subprocess.DEVNULL)
        entries = {}
        with open(cache) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 5:
                    entries[parts[0]] = " ".join(parts[1:5])
    out = os.path.join(HERE, "default.tunecache")
    with open(out, "w") as f:
        for k in sorted(entries):
            f.write(f"{k} {entries[k]}\n")
    print(f"{len(entries)} shapes -> {out}")


if __name__ == "__main__":
    main()
