"""Where an event batch's end-to-end time goes, for a caller choosing how to
hand its arrays to the library.

    python -m xsbench_gb300.e2e_breakdown [--grid unionized|hash|nuclide]
        [--kernel plain|batched] [--size large|small|XL] [--lookups N] [--reps 7]

On one context it times the same lookups eight ways: LCG-sampled on the device
with no outputs, with outputs in device memory and with outputs in page-locked
host memory (xs_run_event); caller samples in device memory with and without
outputs, and caller samples in page-locked host memory with macro_xs and
argmax, argmax only, or no outputs back (xs_lookup_samples). Each line gives
the wall-clock rate of the call, the library's device time and the hash, one
line per case, then a JSON line with the same figures.
"""
from __future__ import annotations

import argparse
import json
import statistics
import time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", default="unionized", choices=["unionized", "hash", "nuclide"])
    ap.add_argument("--kernel", default="plain", choices=["plain", "batched"])
    ap.add_argument("--size", default="large", choices=["small", "large", "XL"])
    ap.add_argument("--lookups", type=int, default=None)
    ap.add_argument("--reps", type=int, default=7)
    a = ap.parse_args(argv)

    import torch

    import xsbench_gb300 as X

    inp = X.make_inputs(size=a.size, grid=a.grid, method="event", lookups=a.lookups)
    n = int(inp.lookups)
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    hE, hM = pin((n,), torch.float64), pin((n,), torch.int32)
    hmacro, hidx = pin((n, 5), torch.float64), pin((n,), torch.uint8)
    dmacro = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    didx = torch.empty(n, dtype=torch.uint8, device="cuda")
    dE = torch.empty(n, dtype=torch.float64, device="cuda")
    dM = torch.empty(n, dtype=torch.int32, device="cuda")
    k = a.kernel
    out = {"grid": a.grid, "kernel": k, "size": a.size, "lookups": n, "cases": {}}
    with X.Context(inp) as ctx:                      # the problem built on the device
        ctx.sample_event(0, n, hE, hM)
        ctx.sample_event(0, n, dE, dM)
        cases = {
            "device samples (LCG), no outputs": lambda: ctx.run_event(kernel=k),
            "device samples (LCG), outputs in device memory":
                lambda: ctx.run_event(macro_out=dmacro, max_idx_out=didx, kernel=k),
            "device samples (LCG), outputs in host memory":
                lambda: ctx.run_event(macro_out=hmacro, max_idx_out=hidx, kernel=k),
            "caller samples in device memory, no outputs":
                lambda: ctx.lookup_samples(dE, dM, kernel=k),
            "caller samples in device memory, outputs in device memory":
                lambda: ctx.lookup_samples(dE, dM, macro_out=dmacro, max_idx_out=didx, kernel=k),
            "caller samples in host memory, macro_xs and argmax to host":
                lambda: ctx.lookup_samples(hE, hM, macro_out=hmacro, max_idx_out=hidx, kernel=k),
            "caller samples in host memory, argmax to host":
                lambda: ctx.lookup_samples(hE, hM, max_idx_out=hidx, kernel=k),
            "caller samples in host memory, no outputs": lambda: ctx.lookup_samples(hE, hM, kernel=k),
        }
        for name, f in cases.items():
            f()
            f()
            wall, dev = [], []
            for _ in range(max(1, a.reps)):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = f()
                wall.append(time.perf_counter() - t0)
                dev.append(r.device_ms)
            w, d = statistics.median(wall), statistics.median(dev) / 1e3
            out["cases"][name] = {"wall_lookups_per_s": n / w, "device_lookups_per_s": n / d,
                                  "wall_ms": w * 1e3, "device_ms": d * 1e3, "hash": r.hash}
            print("%-58s wall %7.1f M/s  device %7.1f M/s  hash %d" % (name, n / w / 1e6, n / d / 1e6,
                                                                       r.hash), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
