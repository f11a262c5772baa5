"""CPU restatement of the learned-guess network (test infrastructure: the oracle for the
gradient check of libeqc's forward and backward kernels; never used by the library).

The network has no counterpart in the reference (thehalfspace/eqcycle starts every CG solve
from the previous displacement, src/main.jl:241).  Layout of the flat parameter vector and
arithmetic follow eqcycle_gb300/csrc/learn.h: four 1-D convolutions (kernel 5, stride 2,
padding 2, 64 channels, GELU), fc1 (GELU), fc2; weights are rounded to BF16 before every
product, sums are carried in FP64 here (FP32 on the GPU).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

C, K, LAYERS, NH, GX, GY = 64, 5, 4, 512, 121, 61


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 value (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def shapes(Nf: int):
    T = [Nf]
    for _ in range(LAYERS):
        T.append((T[-1] - 1) // 2 + 1)
    flat = C * T[-1]
    offs, o = {}, 0
    for l in range(LAYERS):
        cin = 2 if l == 0 else C
        offs[f"cw{l}"] = (o, (C, cin, K)); o += C * cin * K
        offs[f"cb{l}"] = (o, (C,)); o += C
    offs["f1w"] = (o, (NH, flat)); o += NH * flat
    offs["f1b"] = (o, (NH,)); o += NH
    offs["f2w"] = (o, (GX * GY, NH)); o += GX * GY * NH
    offs["f2b"] = (o, (GX * GY,)); o += GX * GY
    return T, flat, offs, o


def unpack(p: np.ndarray, Nf: int, round_bf16: bool = True):
    _, _, offs, n = shapes(Nf)
    assert p.size == n
    out = {}
    for k, (o, shp) in offs.items():
        v = p[o:o + int(np.prod(shp))].reshape(shp)
        is_weight = k.startswith("cw") or k in ("f1w", "f2w")   # biases stay FP32
        out[k] = bf16(v) if (round_bf16 and is_weight) else v.astype(np.float64)
    return out


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _taps(inp_pad, Tout):
    # inp_pad [B, Cin, Tin + 4] -> [K, B, Cin, Tout], tap k reads positions 2t + k
    return np.stack([inp_pad[:, :, k:k + 2 * Tout:2] for k in range(K)])


def forward(p: np.ndarray, x0: np.ndarray, round_bf16: bool = True):
    """x0 [B, 2*Nf] -> (out [B, GX*GY], cache for backward).  round_bf16=False keeps the
    weights in FP64 (finite-difference checks of this restatement itself)."""
    B = x0.shape[0]
    Nf = x0.shape[1] // 2
    T, flat, _, _ = shapes(Nf)
    W = unpack(p, Nf, round_bf16)
    a = x0.reshape(B, 2, Nf).astype(np.float64)
    cache = {"in": [], "z": []}
    for l in range(LAYERS):
        pad = np.pad(a, ((0, 0), (0, 0), (2, 2)))
        taps = _taps(pad, T[l + 1])
        z = np.einsum("oik,kbit->bot", W[f"cw{l}"], taps) + W[f"cb{l}"][None, :, None]
        cache["in"].append(pad)
        cache["z"].append(z)
        a = gelu(z)
    a3 = a.reshape(B, flat)
    zf1 = a3 @ W["f1w"].T + W["f1b"]
    af1 = gelu(zf1)
    out = af1 @ W["f2w"].T + W["f2b"]
    cache.update(a3=a3, zf1=zf1, af1=af1, W=W, T=T, flat=flat, Nf=Nf)
    return out, cache


def loss_and_grad(p: np.ndarray, x0: np.ndarray, tgt: np.ndarray, round_bf16: bool = True):
    """Mean squared error per output and its gradient in the flat parameter layout."""
    out, c = forward(p, x0, round_bf16)
    B, nout = out.shape
    e = out - tgt.astype(np.float64)
    loss = float(np.sum(e * e) / (B * nout))
    g_out = 2.0 * e / (B * nout)
    W, T = c["W"], c["T"]
    _, _, offs, n = shapes(c["Nf"])
    g = np.zeros(n)

    def put(name, val):
        o, shp = offs[name]
        g[o:o + int(np.prod(shp))] = val.reshape(-1)

    put("f2w", g_out.T @ c["af1"])
    put("f2b", g_out.sum(0))
    g_z = (g_out @ W["f2w"]) * gelu_grad(c["zf1"])
    put("f1w", g_z.T @ c["a3"])
    put("f1b", g_z.sum(0))
    g_a = (g_z @ W["f1w"]).reshape(B, C, T[LAYERS])
    for l in range(LAYERS - 1, -1, -1):
        gz = g_a * gelu_grad(c["z"][l])
        pad = c["in"][l]
        taps = _taps(pad, T[l + 1])
        put(f"cw{l}", np.einsum("bot,kbit->oik", gz, taps))
        put(f"cb{l}", gz.sum((0, 2)))
        if l > 0:
            gpad = np.zeros_like(pad)
            for k in range(K):
                gpad[:, :, k:k + 2 * T[l + 1]:2] += np.einsum("oi,bot->bit", W[f"cw{l}"][:, :, k], gz)
            g_a = gpad[:, :, 2:-2]
    return loss, g, out
