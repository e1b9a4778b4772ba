"""Issue cost of FP64-pipe instructions on this GPU: cycles a warp spends per
DFMA, DSETP (FP64 compare) and F2F (double -> float), for 1 to 16 warps of
one CTA per SM and for full and single-lane warps.  Prints one line per case;
the SM's cost per instruction is the warp's over the warps.

    python -m probe.issue
"""
from __future__ import annotations

import ctypes

from probe.build import build

NAMES = {0: "DFMA", 1: "DSETP", 2: "F2F.F32.F64"}


def main() -> None:
    lib = ctypes.CDLL(str(build()))
    lib.nsw6_probe_issue.restype = ctypes.c_double
    lib.nsw6_probe_issue.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    for op in (0, 1, 2):
        for warps in (1, 2, 4, 8, 16):
            for active in (32, 1):
                c = lib.nsw6_probe_issue(op, warps, active, 2000)
                print(f"{NAMES[op]:12s} warps {warps:2d} active lanes {active:2d}: "
                      f"{c:8.2f} cycles per instruction of a warp, {c / warps:7.2f} of the SM", flush=True)


if __name__ == "__main__":
    main()
