"""Algorithmic work per output sample of the response + TDI path.

Used for the roofline figures of the benchmark.  Counts follow the
reference's arithmetic (``LISAResponse.cu:110-207`` interpolation,
``:559-668`` link geometry, ``:300-396`` TDI; orbit interpolation as restated
from lisaanalysistools): every FP64 add, subtract, multiply, divide, square
root and ceil is one operation; each is counted once per output even where the
reference evaluates the same value again (the TDI light travel times).

Bytes are the compulsory DRAM traffic of the two-kernel path: the complex
input read once (16 B), the six link streams written and read once (48 B each
way), the three TDI channels written once (24 B).  Time arrays and tables are
excluded (they are tiny or computable).
"""

from __future__ import annotations


def response_ops_per_link_sample(h: int) -> int:
    """FP64 ops of one (link, sample) projection with h = (order+1)//2."""
    ltt = 1 + 6             # segment t/dt, lerp (hi-lo, /dt, dt*w, t-, *, +)
    x_rec = 1 + 3 * 6       # one segment, three coordinates
    x_em = 1 + 1 + 3 * 6    # t - L, segment, three coordinates
    unit_vector = 3 + 3 + 3 + 1 + 3   # differences, squares, sums, sqrt, divisions
    xi = 6 + 6 + 4 + 1      # u.n, v.n, xi_plus, xi_cross
    dots = 3 * 6            # k.n, k.x_rec, k.x_em
    delays = 2 * 2          # k.x * C_inv, t - ...
    splits = 2 * 6          # (d - t0), *fs, ceil, 1+d, *fs, -
    prefactors = 2 * 8      # eps/deps, ind*deps, -, /deps, 1-frac, 2 mul, add
    interp = 15 + 13 * (h - 1)   # complex: B, D, per tap pair (F, G, 4 div, 2 add,
    #                              2 mul, 2 acc), final 6 per component
    output = 8              # 1 - k.n, reciprocal, 2 sub, 2 mul, add, mul
    return ltt + x_rec + x_em + unit_vector + xi + dots + delays + splits + prefactors + \
        2 * interp + output


def tdi_ops_per_sample(h: int, num_units: int, num_delay_links: int) -> int:
    """FP64 ops of all TDI units of one sample; num_delay_links counts the
    link entries that subtract a light travel time (the -11 markers excluded)."""
    ltt = 1 + 6 * 6          # L(t) of the six links (one shared segment)
    per_unit = 6 + 8 + (9 + 8 * (h - 1)) + 2   # split, prefactor, real interp, sign, add
    return ltt + num_units * per_unit + num_delay_links


def ops_per_sample(order: int, num_units: int, num_delay_links: int) -> dict:
    h = (order + 1) // 2
    resp = 6 * response_ops_per_link_sample(h)
    tdi = tdi_ops_per_sample(h, num_units, num_delay_links)
    return {"response": resp, "tdi": tdi, "total": resp + tdi}


BYTES_PER_SAMPLE = {
    "response": 16 + 48,   # complex128 in, six float64 links out
    "tdi": 48 + 24,        # six links in, three channels out
}
BYTES_PER_SAMPLE["total"] = BYTES_PER_SAMPLE["response"] + BYTES_PER_SAMPLE["tdi"]
