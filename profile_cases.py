"""Profiling harness: runs one named workload a fixed number of times so that
an ncu capture has a short, deterministic launch sequence.

  python profile_cases.py CASE [--n N] [--iters K] [--variant V]

Cases: sort-kv (u32 keys + u32 values), sort-keys (u32 keys; both take
--variant V to run digit-pass variant V), sort-kv64
(u64 keys + u32 values), scan-i32 (exclusive, int64 total), reduce-i32,
hist-u8 (256 bins), segsort-u64kv (lognormal segments, median 256, sigma 2,
n = total keys), rbk-u64 (reduce_by_key over sorted keys with runs, fused
65,536-bin histogram), copy-if-i32 ("x > 0"), transform-u32f32 ("x * 0.18f +
32.0f", uint -> float), transform2-u32 ("x + y"), learned-f32 (learned-CDF
sort of float32 keys: 75% from 8 Gaussians with means in [-1e3, 1e3] and
sigmas log-uniform in [1e-2, 1e2], 20% lognormal(0, 2), 5% copies of 1,000 of
those values, shuffled), bitpack-u32 (delta-coded compression of slowly
increasing timestamps, then decompression), map-u32 (static_map: clear,
insert n distinct keys into 2n slots, find n keys of which half are
absent). Inputs are seeded synthetic
data generated on the device; every call goes through the C ABI on the
library's stream.
"""
from __future__ import annotations

import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "opencl-sdk_gb300"))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--n", type=int, default=1 << 25)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--variant", type=int, default=-1,
                    help="sort cases: the digit-pass variant to use (tuning-table entry for this size)")
    args = ap.parse_args()

    import numpy as np
    import torch

    import gbcompute as gbc

    ctx = gbc.Context(0)
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    n = args.n

    def u32(count):
        return torch.randint(0, 2**32, (count,), dtype=torch.int64, device="cuda", generator=g).to(torch.int32)

    if args.case in ("sort-kv", "sort-keys"):
        k, ko = u32(n), torch.empty(n, dtype=torch.int32, device="cuda")
        v, vo = torch.arange(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")
        kv = args.case == "sort-kv"

        if args.variant >= 0:
            ctx.tuning_set(gbc.tuning_sort_key(4, kv, n), args.variant)

        def step():
            gbc.sort_raw(ctx, k.data_ptr(), ko.data_ptr(), np.uint32, n, v.data_ptr() if kv else 0,
                         vo.data_ptr() if kv else 0)
    elif args.case == "sort-kv64":
        k = torch.randint(-2**63, 2**63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g)
        ko = torch.empty_like(k)
        v, vo = torch.arange(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")

        def step():
            gbc.sort_raw(ctx, k.data_ptr(), ko.data_ptr(), np.uint64, n, v.data_ptr(), vo.data_ptr())
    elif args.case == "scan-i32":
        x = torch.randint(-1000, 1001, (n,), dtype=torch.int32, device="cuda", generator=g)
        y = torch.empty_like(x)
        t = torch.zeros(1, dtype=torch.int64, device="cuda")

        def step():
            gbc.scan_raw(ctx, x.data_ptr(), y.data_ptr(), n, np.int32, exclusive=True, total_device=t.data_ptr())
    elif args.case == "reduce-i32":
        x = torch.randint(-1000, 1001, (n,), dtype=torch.int32, device="cuda", generator=g)
        xb = gbc.DeviceBuffer.wrap(ctx, x.data_ptr(), n, np.int32)

        def step():
            gbc.reduce(ctx, xb)
    elif args.case == "hist-u8":
        x = torch.randint(0, 256, (n,), dtype=torch.uint8, device="cuda", generator=g)
        h = torch.empty(256, dtype=torch.int32, device="cuda")

        def step():
            gbc.histogram_even_raw(ctx, x.data_ptr(), n, np.uint8, h.data_ptr(), 256, 0.0, 256.0)
    elif args.case == "segsort-u64kv":
        rng = np.random.default_rng(4)
        lens = []
        total = 0
        while total < n:
            ln = int(min(max(round(rng.lognormal(np.log(256), 2.0)), 1), 1 << 20))
            ln = min(ln, n - total)
            lens.append(ln)
            total += ln
        offs = np.zeros(len(lens) + 1, dtype=np.int64)
        np.cumsum(lens, out=offs[1:])
        off = torch.from_numpy(offs.astype(np.int32)).cuda()
        k = torch.randint(-2**63, 2**63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g)
        ko = torch.empty_like(k)
        v, vo = torch.arange(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")

        def step():
            gbc.segmented_sort_raw(ctx, k.data_ptr(), ko.data_ptr(), np.uint64, n, off.data_ptr(), len(lens),
                                   v.data_ptr(), vo.data_ptr())
    elif args.case == "rbk-u64":
        # sorted keys with runs of geometric length (mean 40), values < 2^16
        runs = torch.rand(n, device="cuda", generator=g) < 1.0 / 40
        k = torch.cumsum(runs.to(torch.int64), 0) * 2654435761
        v = torch.randint(0, 1 << 16, (n,), dtype=torch.int32, device="cuda", generator=g)
        uk, sums = torch.empty_like(k), torch.empty(n, dtype=torch.int64, device="cuda")
        cnt, h = torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(65536, dtype=torch.int32, device="cuda")

        def step():
            gbc.reduce_by_key_raw(ctx, k.data_ptr(), np.uint64, v.data_ptr(), n, uk.data_ptr(), sums.data_ptr(),
                                  cnt.data_ptr(), h.data_ptr(), want_count=False)
    elif args.case == "copy-if-i32":
        x = torch.randint(-1000, 1001, (n,), dtype=torch.int32, device="cuda", generator=g)
        y = torch.empty_like(x)
        xb = gbc.DeviceBuffer.wrap(ctx, x.data_ptr(), n, np.int32)
        yb = gbc.DeviceBuffer.wrap(ctx, y.data_ptr(), n, np.int32)

        def step():
            gbc.copy_if(ctx, xb, yb, "x > 0")
    elif args.case in ("transform-u32f32", "transform2-u32"):
        x, y = u32(n), u32(n)
        o = torch.empty(n, dtype=torch.int32, device="cuda")
        xb = gbc.DeviceBuffer.wrap(ctx, x.data_ptr(), n, np.uint32)
        yb = gbc.DeviceBuffer.wrap(ctx, y.data_ptr(), n, np.uint32)
        ob = gbc.DeviceBuffer.wrap(ctx, o.data_ptr(), n, np.float32 if args.case == "transform-u32f32" else np.uint32)

        def step():
            if args.case == "transform-u32f32":
                gbc.transform(ctx, xb, ob, "x * 0.18f + 32.0f")
            else:
                gbc.transform(ctx, xb, yb, ob, "x + y")
    elif args.case == "learned-f32":
        n75, n20 = int(0.75 * n), int(0.20 * n)
        means = torch.rand(8, device="cuda", generator=g, dtype=torch.float64) * 2e3 - 1e3
        sig = torch.exp((torch.rand(8, device="cuda", generator=g, dtype=torch.float64) * 2 - 1) * np.log(100.0))
        comp = torch.randint(0, 8, (n75,), device="cuda", generator=g)
        a = (means[comp] + sig[comp] * torch.randn(n75, device="cuda", generator=g, dtype=torch.float64)).float()
        b = torch.exp(2.0 * torch.randn(n20, device="cuda", generator=g))
        pool = torch.cat([a[:500], b[:500]])
        c = pool[torch.randint(0, 1000, (n - n75 - n20,), device="cuda", generator=g)]
        k = torch.cat([a, b, c])[torch.randperm(n, device="cuda", generator=g)].contiguous()
        del a, b, c, comp
        ko = torch.empty_like(k)

        def step():
            gbc.sort_learned(ctx, k.data_ptr(), ko.data_ptr(), np.float32, n)
    elif args.case == "bitpack-u32":
        # slowly increasing timestamps, delta coding, 2,048-element chunks:
        # compress, then decompress the result
        steps = torch.randint(0, 50, (n,), dtype=torch.int64, device="cuda", generator=g)
        ts = ((1700000000 + torch.cumsum(steps, 0)) & 0xFFFFFFFF).to(torch.int32)
        cap = gbc.bitpack_words_bound(n, 2048)
        packed = torch.empty(cap, dtype=torch.int32, device="cuda")
        back = torch.empty_like(ts)

        def step():
            w = gbc.compress_bitpack_raw(ctx, ts.data_ptr(), n, packed.data_ptr(), cap, delta=True)
            gbc.decompress_bitpack_raw(ctx, packed.data_ptr(), w, n, back.data_ptr(), delta=True)
    elif args.case == "map-u32":
        # n distinct keys into 2n slots, then n finds (half absent)
        mk = ((torch.arange(n, dtype=torch.int64, device="cuda") * 2654435761 + 12345) & 0xFFFFFFFE).to(torch.int32)
        mv = torch.arange(n, dtype=torch.int32, device="cuda")
        qk = mk.clone()
        qk[1::2] |= 1
        got = torch.empty_like(mv)
        smap = gbc.StaticMap(ctx, 2 * n)

        def step():
            smap.clear()
            smap.insert_raw(mk.data_ptr(), mv.data_ptr(), n)
            smap.find_raw(qk.data_ptr(), n, got.data_ptr())
    else:
        raise SystemExit(f"unknown case {args.case}")

    torch.cuda.synchronize()
    for _ in range(args.iters):
        step()
    ctx.finish()
    print(f"{args.case}: {args.iters} iterations of n={n} done")
    ctx.close()


if __name__ == "__main__":
    main()
