"""Study (not on the engine's path): NMSE of the learned estimator against its receptive field.

    python -m hermespy_gb300.study_receptive_field --pairs 300000 --out receptive_field.json

The shipped network (six 3x3 layers, 32 channels, residual over the per-stream LS
estimate) sees 13 x 13 grid elements around each output, while the tap-domain LMMSE
estimator it is judged against combines every pilot of the frame. This study trains
the same architecture with dilated layers (the same six layers, 32 channels and 3x3
taps, spread over the grid) on the same simulator pairs, and reports the validation
NMSE of each next to per-stream LS and the tap-domain LMMSE estimator (the genie one,
with the channel's delays, powers and Doppler). The engine's CNN kernels implement
the specified undilated 3x3 form; the variants here run as PyTorch convolutions, since
the question is the architecture's, not the kernels'.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch
import torch.nn.functional as F

from .learned import PairSource, random_channels
from .train_estimator import FS, engines_for, evaluate, pilot_waveform, workload_channel

# name: per-layer dilation (rows = words, columns = subcarriers)
VARIANTS = {
    "3x3 (shipped form)": [(1, 1)] * 6,
    "columns 1-32": [(1, 1), (1, 2), (1, 4), (1, 8), (1, 16), (1, 32)],
    "rows 1-2, columns 1-32": [(1, 1), (2, 2), (2, 4), (1, 8), (1, 16), (1, 32)],
    "columns 1-81": [(1, 1), (1, 3), (1, 9), (1, 27), (1, 81), (1, 1)],
}


def receptive_field(dil) -> tuple[int, int]:
    return 1 + 2 * sum(d[0] for d in dil), 1 + 2 * sum(d[1] for d in dil)


class DilatedCnn(torch.nn.Module):
    """x0 = LS / s (32 channels: 16 pairs x re, im), h_l = relu(conv_l(h_{l-1})), out = LS + s conv_6(h_5),
    s = RMS of the drop's LS estimate: the engine's network with dilated taps."""

    def __init__(self, dil, seed: int) -> None:
        super().__init__()
        g = torch.Generator().manual_seed(seed)
        self.dil = dil
        self.w = torch.nn.ParameterList()
        self.b = torch.nn.ParameterList()
        for i in range(6):
            std = math.sqrt(2.0 / (32 * 9)) * (0.1 if i == 5 else 1.0)
            self.w.append(torch.nn.Parameter(torch.randn(32, 32, 3, 3, generator=g) * std))
            self.b.append(torch.nn.Parameter(torch.zeros(32)))

    def forward(self, ls: torch.Tensor) -> torch.Tensor:
        B, W, C = ls.shape[0], ls.shape[-2], ls.shape[-1]
        z = torch.view_as_real(ls.reshape(B, 16, W, C)).permute(0, 1, 4, 2, 3).reshape(B, 32, W, C)
        s = torch.sqrt(torch.mean(z * z, dim=(1, 2, 3), keepdim=True) * 2.0).clamp_min(1e-30)
        h = (z / s).to(torch.bfloat16)
        for i, (dh, dw) in enumerate(self.dil):
            h = F.conv2d(h, self.w[i].to(torch.bfloat16), self.b[i].to(torch.bfloat16), padding=(dh, dw),
                         dilation=(dh, dw))
            if i < 5:
                h = torch.relu(h)
        out = z + s * h.float()
        out = out.reshape(B, 16, 2, W, C).permute(0, 1, 3, 4, 2).contiguous()
        return torch.view_as_complex(out).reshape(ls.shape)

    def refine(self, csi: torch.Tensor, stream=None) -> torch.Tensor:  # the evaluate() interface
        with torch.no_grad():
            csi.copy_(self.forward(csi))
        return csi


def train_variant(dil, source: PairSource, pairs: int, lr: float, seed: int) -> tuple[DilatedCnn, float]:
    model = DilatedCnn(dil, seed).cuda()
    opt = torch.optim.Adam(model.parameters(), lr=lr)
    steps = max(1, pairs // source.batch)
    t0 = time.perf_counter()
    for s in range(steps):
        ls, truth, _ = source.next()
        for grp in opt.param_groups:
            grp["lr"] = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
        loss = torch.mean(torch.abs(model(ls) - truth) ** 2)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
    torch.cuda.synchronize()
    return model, time.perf_counter() - t0


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=300_000, help="training pairs (drops) per variant")
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--val-drops", type=int, default=256)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    wf = pilot_waveform()
    source = PairSource(wf, FS, random_channels(64, args.seed), args.batch, args.seed)
    work = engines_for(wf, [workload_channel()], 64, 20_000)
    rows = []
    for name, dil in VARIANTS.items():
        model, secs = train_variant(dil, source, args.pairs, args.lr, args.seed)
        val = evaluate(model, work, (0.0, 30.0), args.val_drops, 2)
        rows.append({"variant": name, "dilation": dil, "receptive_field": receptive_field(dil),
                     "nmse_db": val["learned"], "ls_db": val["ls"], "lmmse_db": val["lmmse"], "train_s": secs})
        print(json.dumps(rows[-1]), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"pairs": args.pairs, "rows": rows}, f, indent=1)


if __name__ == "__main__":
    main()
