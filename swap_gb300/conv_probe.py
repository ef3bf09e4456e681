"""Run the surrogate's tensor-core convolution on random BF16 data, for
profiling one launch in isolation:

    python -m swap_gb300.conv_probe CIN COUT NX NY NZ [REPEATS]

CIN, COUT are 16 or 32 (the layer shapes of the network); NX*NY*NZ must be a
multiple of 128, and NX a multiple of 128 selects the line-ring form.
"""
from __future__ import annotations

import sys


def main(argv=None) -> int:
    import torch

    from . import abi

    a = [int(x) for x in (argv if argv is not None else sys.argv[1:])]
    if len(a) not in (5, 6):
        print(__doc__)
        return 2
    cin, cout, nx, ny, nz = a[:5]
    reps = a[5] if len(a) == 6 else 2
    lib = abi.load()
    V = nx * ny * nz
    X = torch.randn(V, cin, device="cuda").to(torch.bfloat16)
    W = (0.1 * torch.randn(27, cout, cin, device="cuda")).to(torch.bfloat16)
    b = torch.zeros(cout, device="cuda")
    Y = torch.empty(V, cout, dtype=torch.bfloat16, device="cuda")
    for _ in range(reps):
        r = lib.swap_conv3_check(nx, ny, nz, cin, cout, X.data_ptr(), W.data_ptr(), b.data_ptr(), Y.data_ptr(), None,
                                 1)
        if r:
            print(f"swap_conv3_check returned {r}")
            return 1
    torch.cuda.synchronize()
    print("ok")
    return 0


if __name__ == "__main__":
    sys.exit(main())
