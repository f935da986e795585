"""Algorithmic work per output sample of the response + TDI path.

Used for the roofline figures of the benchmark.  Counts follow the
reference's arithmetic (``LISAResponse.cu:110-207`` interpolation,
``:559-668`` link geometry, ``:300-396`` TDI; orbit interpolation as restated
from lisaanalysistools) with per-knot constants (the segment slopes) hoisted
and identical subexpressions counted once.  FP64 operations are split into
divide-class operations (division, square root), which the FP64 pipe executes
as multi-instruction sequences, and the rest (add, subtract, multiply, ceil,
conversions), one pipe slot each.

The roofline of the plain path is the FP64 pipe: ``slots = ops + divs * c``
with ``c`` the measured FMA-slots per division (probe kernel), against the
measured FP64 FMA peak.

Bytes are the compulsory DRAM traffic of the two-kernel path: the complex
input read once (16 B), the six link streams written and read once (48 B each
way), the three TDI channels written once (24 B).  Time arrays and tables are
excluded (they are tiny or computable).
"""

from __future__ import annotations


def response_counts(h: int) -> dict:
    """FP64 ops and divide-class ops of one (link, sample) projection."""
    ops = (4          # L(t): t - dt*w, slope*(.) + lo           (+1 div: segment)
           + 6        # x_rec(t): 3 coordinates, shares (t - dt*w)
           + 1 + 8    # t_em = t - L; x_em(t_em)                 (+1 div: segment)
           + 9        # n = x_rec - x_em, |n|^2                  (+1 sqrt, +3 div)
           + 17       # u.n, v.n, xi_plus, xi_cross
           + 18       # k.n, k.x_rec, k.x_em
           + 4        # delays t - k.x * C_inv
           + 2 * 6    # index splits: -t0, *fs, ceil, cvt, 1+d, -
           + 2 * 6    # A(eps) lerp: cvt, ind*deps, -, 1-frac, 2 mul + add  (+2 div each)
           + 2 * (14 + 8 * (h - 1))   # complex interp: B, D, F, G, 2 adds, 2 mul E,
           #                            2 acc per tap pair; 6 per component at the end
           + 7)       # 1 - k.n, 2 sub, 2 mul, add, mul          (+1 div)
    divs = 1 + 1 + 4 + 2 * 2 + 2 * 4 * (h - 1) + 1
    return {"ops": ops, "divs": divs}


def tdi_counts(h: int, num_units: int, num_delay_links: int) -> dict:
    """FP64 ops and divide-class ops of all TDI units of one sample;
    num_delay_links counts the link entries that subtract a light travel time
    (the -11 markers excluded)."""
    ops = (2 + 6 * 2                              # L(t) of the six links (+1 div)
           + num_delay_links                      # delay -= L
           + num_units * (6 + 6 + 8 + 5 * (h - 1) + 2))
    #       split, A lerp, real interp (B, D, final 6; F, G, add, mul E, acc per tap
    #       pair), sign and accumulate
    divs = 1 + num_units * (2 + 2 * (h - 1))
    return {"ops": ops, "divs": divs}


def counts_per_sample(order: int, num_units: int, num_delay_links: int) -> dict:
    h = (order + 1) // 2
    r = response_counts(h)
    t = tdi_counts(h, num_units, num_delay_links)
    return {"response": {"ops": 6 * r["ops"], "divs": 6 * r["divs"]},
            "tdi": t,
            "total": {"ops": 6 * r["ops"] + t["ops"], "divs": 6 * r["divs"] + t["divs"]}}


def fp64_slots(counts: dict, div_cost: float) -> float:
    """FP64-pipe FMA slots of `counts` with a division costing `div_cost` slots."""
    return counts["ops"] + counts["divs"] * div_cost


BYTES_PER_SAMPLE = {
    "response": 16 + 48,   # complex128 in, six float64 links out
    "tdi": 48 + 24,        # six links in, three channels out
}
BYTES_PER_SAMPLE["total"] = BYTES_PER_SAMPLE["response"] + BYTES_PER_SAMPLE["tdi"]


def mixed_index_ops(num_units: int, delay_subtractions: int) -> dict:
    """FP64 operations of the mixed path's exact index path per output sample:
    the work that must stay in FP64 for the integer delays to be bit-exact
    (orbit lerps of L and positions, k.x, delays, index splits), with each
    orbit-segment lookup counted as one operation.  `delay_subtractions` is the
    number of TDI partial sums evaluated per sample (prefix sharing included).
    Taps, weights and projections run on the FP32 pipe and are not counted."""
    per_link = (1 + 4      # segment(t), L(t)
                + 6        # x_rec: 3 coordinates
                + 1 + 1 + 8  # t_em, segment(t_em), x_em
                + 2 * 6    # k.x_rec, k.x_em
                + 2 * 2    # delays
                + 2 * 6)   # index splits
    response = 6 * per_link
    tdi = 1 + 6 * 2 + delay_subtractions + num_units * 6
    return {"response": response, "tdi": tdi, "total": response + tdi}


def prefix_shared_subtractions(delay_lists) -> int:
    """Partial sums evaluated when each unit reuses the common prefix of the
    previous unit's delay list (delay_lists: sequence of link sequences)."""
    total, prev = 0, []
    for cur in delay_lists:
        keep = 0
        while keep < min(len(cur), len(prev)) and cur[keep] == prev[keep]:
            keep += 1
        total += len(cur) - keep
        prev = cur
    return total


def mixed_index_ops_grouped(num_groups: int, max_len: int) -> dict:
    """FP64 operations of the exact index path per output sample in the mixed
    kernel's equal-arm form, counted as in :func:`mixed_index_ops`: all six
    light travel times are one value, every link leaving a spacecraft has the
    same emission time, so a sample needs three receiver sides and three
    emitter sides (not six links), and the TDI units of one delay-list length
    share one delay and one index split (`num_groups` lengths, partial sums up
    to `max_len` links)."""
    receiver = (1          # segment(t)
                + 6        # x_rec: 3 coordinates
                + 6        # k.x_rec
                + 2        # delay
                + 6)       # index split
    emitter = (4           # L(t) (the receiver's segment)
               + 1 + 1 + 8  # t_em, segment(t_em), x_em
               + 6         # k.x_em
               + 2         # delay
               + 6)        # index split
    response = 3 * receiver + 3 * emitter
    tdi = 1 + 2 + max_len + num_groups * 6
    return {"response": response, "tdi": tdi, "total": response + tdi}
