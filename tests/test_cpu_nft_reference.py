"""The NFT transport's CPU-side pins (no GPU): the reference's NFT code compiled from its
sources (oracle/_ref/libref_nft.so, where the sources are present) against the committed
fixtures, the window split the GPU tests use against the reference's own window driver,
and the group-array layout the GPU entry point assumes."""
import os
import platform
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(HERE, "golden"))

import simstack_gb300 as sg  # noqa: E402
from oracle import oracle as O  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "nft_transport.npz"))
needs_ref = pytest.mark.skipif(not O.ref_nft_available(), reason="oracle/_ref/libref_nft.so not built (no reference sources)")


def test_fixture_cases_complete():
    cases = {k.split("/")[0] for k in G.files}
    assert {"run600", "edge_one_cell", "edge_last_cell_site", "edge_site_beyond", "edge_stride0", "edge_no_sites",
            "edge_denormal"} <= cases
    for c in cases:
        for mode in ("ftz", "ieee"):
            for n in ("rows", "hot", "sites", "out_sum", "evap_kg"):
                assert f"{c}/{mode}_{n}" in G.files
    # a site row beyond the channel: the reference applies no site at all
    assert not G["edge_site_beyond/ftz_sites"].reshape(-1, 288)[:, 216:].any()
    # stride 0: only the last site (counted down first) is applied
    removed = G["edge_stride0/ftz_sites"].reshape(-1, 288)[:, 216 + 8:]
    assert not removed[:-1].any() and removed[-1].any()


@needs_ref
def test_group_layout_matches_the_entry_point():
    lay = O.ref_nft_layout()
    assert lay["lanes"] == sg.NFT_LANES and lay["fields"] == sg.NFT_FIELDS
    for name, key in (("rows", "row_bytes"), ("hot", "hot_bytes"), ("cold", "cold_bytes"), ("sites", "site_bytes")):
        assert lay[key] == 4 * sg.NFT_FLOATS[name], name
    # field offsets the kernel reads (floats): hot c/kT/bT/ko, cold kw/kr/ge/ev, site drop/removed
    assert [lay[k] // 4 for k in ("hot_c", "hot_kT", "hot_bT", "hot_ko")] == [0, 8, 16, 24]
    assert [lay[k] // 4 for k in ("cold_kw", "cold_kr", "cold_ge", "cold_ev")] == [24, 32, 40, 48]
    assert [lay[k] // 4 for k in ("site_drop", "site_removed")] == [16, 216]


@needs_ref
def test_split_window_equals_reference_driver():
    """prepare / transport / finish reaches nft_run<f32x8>'s state (30 windows)."""
    a, b = O.RefNftSystem(12), O.RefNftSystem(12)
    a.run(30)
    for _ in range(30):
        b.prepare()
        b.transport()
        b.finish()
    assert a.digest() == b.digest()


@needs_ref
@pytest.mark.parametrize("case", ["edge_one_cell", "edge_last_cell_site", "edge_site_beyond", "edge_stride0",
                                  "edge_no_sites", "edge_denormal"])
def test_fixtures_reproduce_on_this_host(case):
    """The reference's transport run here gives the committed bits: IEEE on any host, FTZ/DAZ
    where the reference sets it (x86-64)."""
    import make_nft_golden as M

    c = {k.split("/", 1)[1]: G[k] for k in G.files if k.startswith(case + "/")}
    meta = {k: int(c[k]) for k in ("groups", "cells", "sites", "site_offset", "site_stride", "substeps")}
    before = {n: c[f"in_{n}"] for n in M.ARRAYS}
    modes = ["ieee"] + (["ftz"] if platform.machine() in ("x86_64", "AMD64") else [])
    for mode in modes:
        got = M.transport_groups(before, meta["groups"], meta["cells"], meta["sites"], meta["site_offset"],
                                 meta["site_stride"], c["ref"], c["env"], meta["substeps"], mode == "ieee")
        for n in M.OUTPUTS:
            assert got[n].tobytes() == c[f"{mode}_{n}"].tobytes(), (mode, n)
