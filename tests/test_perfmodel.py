"""The work model behind the benchmark's roofline figures: per-sample FP64
operation counts of the plain path and of the mixed path's exact index path,
on the reference's 1st/2nd-generation TDI tables."""

import numpy as np

from fastlisaresponse_gb300 import perfmodel as pm
from fastlisaresponse_gb300.response import (NO_LINK, TDI_FIRST_GENERATION,
                                              TDI_SECOND_GENERATION_EXTRA, tdi_unit_tables)


def _tables(gen):
    combos = list(TDI_FIRST_GENERATION)
    if gen == 2:
        combos += TDI_SECOND_GENERATION_EXTRA
    t = tdi_unit_tables(combos)
    links = t["tdi_link_combinations"]
    lists = []
    for u in range(t["num_units"]):
        s, n = t["unit_starts"][u], t["unit_lengths"][u]
        lists.append([x for x in links[s:s + n].tolist() if x != NO_LINK])
    return t["num_units"], int(np.sum(links != NO_LINK)), lists


def test_plain_path_counts_order_25():
    assert pm.response_counts(13) == {"ops": 318, "divs": 107}
    units, delay_links, _ = _tables(2)
    assert (units, delay_links) == (48, 168)
    assert pm.tdi_counts(13, units, delay_links) == {"ops": 4118, "divs": 1249}
    total = pm.counts_per_sample(25, units, delay_links)["total"]
    assert total == {"ops": 6 * 318 + 4118, "divs": 6 * 107 + 1249}
    # one division weighted as 7.5 FMA slots (the measured GB300 ratio)
    assert pm.fp64_slots({"ops": 10, "divs": 2}, 7.5) == 25.0


def test_mixed_index_path_counts():
    for gen, units, subtractions, total in ((1, 24, 18, 469), (2, 48, 60, 655)):
        n_units, _, lists = _tables(gen)
        assert n_units == units
        assert pm.prefix_shared_subtractions(lists) == subtractions
        assert pm.mixed_index_ops(units, subtractions)["total"] == total


def test_prefix_sharing_and_bytes():
    assert pm.prefix_shared_subtractions([[12], [12, 21], [13], [13, 31, 12]]) == 1 + 1 + 1 + 2
    assert pm.prefix_shared_subtractions([]) == 0
    assert pm.BYTES_PER_SAMPLE == {"response": 64, "tdi": 72, "total": 136}


def test_mixed_index_path_counts_equal_arms():
    """Equal arms: three receiver and three emitter sides per sample, one
    split per delay-list length (8 lengths up to 7 links in 2nd generation)."""
    _, _, lists = _tables(2)
    lens = {len(x) for x in lists}
    assert (len(lens), max(lens)) == (8, 7)
    got = pm.mixed_index_ops_grouped(len(lens), max(lens))
    assert got == {"response": 3 * 21 + 3 * 28, "tdi": 3 + 7 + 48, "total": 205}
