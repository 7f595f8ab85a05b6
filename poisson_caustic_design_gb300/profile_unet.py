"""Fixed workloads of the learned warm start's kernels, for timing and for
profiler captures (each run is deterministic and small enough for a
full-metric capture of a few launches).

    python -m poisson_caustic_design_gb300.profile_unet gemm [--time] [--paths 2,3,1]
        the GEMM on three U-Net contraction shapes (M x N x K): 131072 x 32 x
        288 (first 32->32 conv at 64^2 x 32), 32768 x 64 x 576 (64->64 conv at
        32^2 x 32), 16384 x 256 x 2304 (bottom 256->256 conv at 32^2 x 16), one
        launch per shape and path (2: tcgen05, 1: mma.sync, 9: torch.matmul as
        a timing reference; default 2); --shape M,N,K replaces the shapes; with --time, CUDA-event medians
        (L2 flushed between launches)
    python -m poisson_caustic_design_gb300.profile_unet conv [--time]
        the 3x3 convolution as an implicit GEMM on the tcgen05 kernel (no
        im2col; 4-D TMA boxes of the NHWC input per tap) on two U-Net layers:
        32 -> 32 channels at 256^2 x 16 and 128 -> 128 at 64^2 x 16, one launch
        each; with --time, CUDA-event medians (L2 flushed) beside torch's
        conv2d on the same BF16 data (cuDNN, NCHW channels-last, a timing
        reference only)
    python -m poisson_caustic_design_gb300.profile_unet train R B STEPS [--path P]
        STEPS training steps of a resolution-R network on batch B (seeded
        random inputs); with --time, the CUDA-event mean of the steps after the
        first (--path 1 pins the GEMMs to the mma.sync kernel)
"""
import argparse
import json
import os
import sys

SHAPES = ((131072, 32, 288), (32768, 64, 576), (16384, 256, 2304))


def _median_ms(fn, reps=20):
    import torch

    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ts.sort()
    return ts[len(ts) // 2]


def gemm(timed: bool, paths=(2,), shapes=SHAPES) -> dict:
    import torch

    from . import _lib

    L = _lib.load()
    out = {}
    for M, N, K in shapes:
        g = torch.Generator(device="cpu").manual_seed(M + N + K)
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
        C = torch.empty(M, N, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        for path in paths:
            if path == 9:  # cuBLAS through torch (BF16 out), a timing reference only
                def run():
                    torch.matmul(A, B.T)
            else:
                def run():
                    st = L.pcd_gemm_bf16_path(A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N, M, N, K, 1, None, path,
                                              s)
                    if st != 0:
                        raise RuntimeError(L.pcd_last_error())

            run()
            torch.cuda.synchronize()
            if path == 9:
                out[f"{M}x{N}x{K}_torch_ms"] = _median_ms(run) if timed else None
                continue
            ref = A.float() @ B.float().T
            err = (C - ref).abs().max().item() / ref.abs().max().item()
            if err > 1e-5 * max(1.0, (K / 1024) ** 0.5):  # FP32 sums in another order drift with sqrt(K)
                raise RuntimeError(f"{M}x{N}x{K} path {path}: relative error {err}")
            if timed:
                ms = _median_ms(run)
                out[f"{M}x{N}x{K}_path{path}"] = {"ms": ms, "tflops": 2.0 * M * N * K / ms / 1e9}
    if L.pcd_gemm_bf16_status() != 0:
        raise RuntimeError(L.pcd_last_error())
    return out


CONVS = ((16, 256, 256, 32, 32), (16, 64, 64, 128, 128))  # batch, height, width, Cin, Cout


def conv(timed: bool) -> dict:
    import torch
    import torch.nn.functional as F

    from . import _lib

    L = _lib.load()
    out = {}
    for B, H, W, C, N in CONVS:
        g = torch.Generator(device="cpu").manual_seed(B + H + C)
        x = torch.randn(B, H, W, C, generator=g).to(torch.bfloat16).cuda()
        w = torch.randn(N, 9 * C, generator=g).to(torch.bfloat16).cuda()
        y = torch.empty(B * H * W, N, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream

        def run():
            st = L.pcd_conv3x3_bf16(x.data_ptr(), B, H, W, C, C, w.data_ptr(), 9 * C, N, y.data_ptr(), N, s)
            if st != 0:
                raise RuntimeError(L.pcd_last_error())

        run()
        torch.cuda.synchronize()
        xt = x.permute(0, 3, 1, 2)  # NCHW view of the NHWC data (channels-last)
        wt = w.reshape(N, 3, 3, C).permute(0, 3, 1, 2).contiguous(memory_format=torch.channels_last)
        ref = F.conv2d(xt.float(), wt.float(), padding=1).permute(0, 2, 3, 1).reshape(B * H * W, N)
        err = (y - ref).abs().max().item() / ref.abs().max().item()
        if err > 1e-5:
            raise RuntimeError(f"conv {B}x{H}x{W}x{C}->{N}: relative error {err}")
        key = f"{B}x{H}x{W}_{C}to{N}"
        if timed:
            ms = _median_ms(run)
            tms = _median_ms(lambda: F.conv2d(xt, wt, padding=1))
            out[key] = {"ms": ms, "tflops": 2.0 * B * H * W * N * 9 * C / ms / 1e9, "torch_ms": tms,
                        "bytes_in_out": B * H * W * (2 * C + 4 * N)}
    if L.pcd_gemm_bf16_status() != 0:
        raise RuntimeError(L.pcd_last_error())
    return out


def train(R: int, B: int, steps: int, path: int, timed: bool) -> dict:
    import torch

    from . import Context, learned

    ctx = Context(0)
    net = learned.UNet(ctx, resolution=R, max_batch=B, seed=1)
    L = net._L
    if L.pcd_gemm_set_default_path(path) != 0:
        raise RuntimeError(L.pcd_last_error())
    g = torch.Generator(device="cpu").manual_seed(R + B)
    x = torch.randn(B, R, R, generator=g).cuda()
    t = torch.randn(B, R, R, generator=g).cuda()
    loss = net.train_step(x, t, 1e-4)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps - 1):
        loss = net.train_step(x, t, 1e-4)
    e1.record()
    torch.cuda.synchronize()
    out = {"resolution": R, "batch": B, "loss": loss, "path": path}
    if timed and steps > 1:
        out["ms_per_step"] = e0.elapsed_time(e1) / (steps - 1)
    L.pcd_gemm_set_default_path(0)
    net.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="what", required=True)
    a = sub.add_parser("gemm")
    a.add_argument("--time", action="store_true")
    a.add_argument("--paths", default="2")
    a.add_argument("--shape", action="append", default=None, help="M,N,K (repeatable; default the three shapes)")
    c = sub.add_parser("conv")
    c.add_argument("--time", action="store_true")
    b = sub.add_parser("train")
    b.add_argument("R", type=int)
    b.add_argument("B", type=int)
    b.add_argument("steps", type=int)
    b.add_argument("--path", type=int, default=0)
    b.add_argument("--time", action="store_true")
    args = ap.parse_args(argv)
    if args.what == "conv":
        res = conv(args.time)
    elif args.what == "gemm":
        shapes = tuple(tuple(int(v) for v in s.split(",")) for s in args.shape) if args.shape else SHAPES
        res = gemm(args.time, tuple(int(p) for p in args.paths.split(",")), shapes)
    else:
        res = train(args.R, args.B, args.steps, args.path, args.time)
    print(json.dumps(res))


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
