"""The C ABI library: loads without a GPU, exports every declared symbol,
its ctypes mirror matches the C layout, and its host-side parsers follow
the reference's rules (checked against the oracle and the golden vectors)."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import port
from spinterps_gb300 import _native as nat

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        names.update(re.findall(r"^(?:int|int64_t|const char \*)\s*(spi_\w+)\s*\(", txt, re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = nat.load()
    decl = declared_symbols()
    assert decl, "no declarations found"
    for name in decl:
        assert hasattr(lib, name), name
    assert sorted(decl) == nat.EXPORTS
    assert lib.spi_version().startswith(b"spinterps_gb300")


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "spinterps_gb300.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  printf("spi_vg_t %zu\nspi_domain_t %zu\nspi_systems_t %zu\nspi_out_t %zu\n",
         sizeof(spi_vg_t), sizeof(spi_domain_t), sizeof(spi_systems_t), sizeof(spi_out_t));
  printf("spi_krige_ws_t %zu\n", sizeof(spi_krige_ws_t));
  P(spi_krige_ws_t, cell_yy) P(spi_krige_ws_t, tier)
  P(spi_vg_t, sill) P(spi_vg_t, range) P(spi_domain_t, n_drift) P(spi_domain_t, min_vg_val)
  P(spi_domain_t, stn_split) P(spi_domain_t, cell_split) P(spi_domain_t, split_res)
  P(spi_systems_t, max_n)
  P(spi_systems_t, out_row) P(spi_out_t, clip_min) P(spi_out_t, clip_max)
  return 0;
}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run(
        [str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    assert int(got["spi_vg_t"]) == ctypes.sizeof(nat.VgT)
    assert int(got["spi_domain_t"]) == ctypes.sizeof(nat.DomainT)
    assert int(got["spi_systems_t"]) == ctypes.sizeof(nat.SystemsT)
    assert int(got["spi_out_t"]) == ctypes.sizeof(nat.OutT)
    assert int(got["spi_krige_ws_t"]) == ctypes.sizeof(nat.KrigeWsT)
    assert int(got["spi_krige_ws_t.cell_yy"]) == nat.KrigeWsT.cell_yy.offset
    assert int(got["spi_krige_ws_t.tier"]) == nat.KrigeWsT.tier.offset
    assert int(got["spi_vg_t.sill"]) == nat.VgT.sill.offset
    assert int(got["spi_vg_t.range"]) == nat.VgT.range.offset
    assert int(got["spi_domain_t.n_drift"]) == nat.DomainT.n_drift.offset
    assert int(got["spi_domain_t.min_vg_val"]) == nat.DomainT.min_vg_val.offset
    assert int(got["spi_domain_t.stn_split"]) == nat.DomainT.stn_split.offset
    assert int(got["spi_domain_t.cell_split"]) == nat.DomainT.cell_split.offset
    assert int(got["spi_domain_t.split_res"]) == nat.DomainT.split_res.offset
    assert int(got["spi_systems_t.max_n"]) == nat.SystemsT.max_n.offset
    assert int(got["spi_systems_t.out_row"]) == nat.SystemsT.out_row.offset
    assert int(got["spi_out_t.clip_min"]) == nat.OutT.clip_min.offset
    assert int(got["spi_out_t.clip_max"]) == nat.OutT.clip_max.offset


def _parse(s):
    v = nat.VgT()
    rc = nat.lib().spi_parse_vg(s.encode(), ctypes.byref(v))
    return rc, v


def test_parse_vg_matches_reference_rules(golden):
    for s in list(golden["k_vgs"]) + ["1.0 Nug(0.0)", "0.3 Gau(-5)", "2 Exp(1e5)",
                                      " 0.5 Sph(300) +0.5 Exp(10) "]:
        s = str(s)
        rc, v = _parse(s)
        assert rc == 0, s
        ref = port.parse_vg_str(s)
        assert v.n_comp == len(ref)
        for k, (code, sill, rng) in enumerate(ref):
            assert v.code[k] == code and v.sill[k] == sill and v.range[k] == rng, s


@pytest.mark.parametrize("bad", ["1.0 Foo(3)", "1.0  Exp(3)", "1.0 Exp3", "Exp(3)",
                                 "1.0 Exp(3) + ", "x Exp(3)", "1.0 Exp(1e+5)"])
def test_parse_vg_rejects_what_the_reference_rejects(bad):
    rc, _ = _parse(bad)
    assert rc == 2  # SPI_ERR_VG
    with pytest.raises(Exception):
        port.parse_vg_str(bad)


def test_parse_vg_too_many_components():
    rc, _ = _parse(" + ".join(["0.1 Exp(10)"] * 5))
    assert rc == 5  # SPI_ERR_TOO_LARGE


def test_nuggetness_matches_reference(golden):
    for s, r4, r0 in zip(golden["k_nug_strs"], golden["k_nug_1e-4"], golden["k_nug_0"]):
        for mvv, r in ((1e-4, r4), (0.0, r0)):
            out = nat.c_i32(-1)
            assert nat.lib().spi_check_full_nuggetness(str(s).encode(), mvv, ctypes.byref(out)) == 0
            assert bool(out.value) == bool(r), (s, mvv)


def test_null_and_size_errors_without_gpu():
    lib = nat.lib()
    assert lib.spi_fill_dists_2d_mat(None, None, -1, None, None, 3, None, None) == 1
    assert lib.spi_fill_dists_2d_mat(None, None, 0, None, None, 0, None, None) == 0
    assert lib.spi_parse_vg(None, None) == 1
    out = nat.OutT()
    assert lib.spi_fill_rows(-1, None, None, None, 10, ctypes.byref(out), None) == 1
    dom = nat.DomainT()
    dom.n_drift = 99
    sy = nat.SystemsT()
    sy.n_sys = 1
    ws = nat.KrigeWsT()
    assert lib.spi_krige_factor(ctypes.byref(dom), ctypes.byref(sy), ctypes.byref(ws), 1e12,
                                None) == 5
    dom.n_drift = 0
    assert lib.spi_krige_factor(ctypes.byref(dom), ctypes.byref(sy), ctypes.byref(ws), 1e12,
                                None) == 1  # null workspace arrays
    dom.n_cells = 10
    assert lib.spi_krige_cells(ctypes.byref(dom), ctypes.byref(sy), None, ctypes.byref(ws), 1,
                               1, 2, 1e8, ctypes.byref(out), None) == 1


def test_host_mirror_has_no_cpu_fallback():
    import torch
    import spinterps_gb300 as spi
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from spinterps_gb300 import driver, fitvgs, nebs, steps, warmstart
    x, y, z = np.array([0.0, 1e3, 2e3]), np.array([0.0, 5e2, 2e3]), np.array([[1.0, 2.0, 3.0]])
    calls = {
        "interp_steps": lambda: spi.interp_steps(x, y, z, x[:2], y[:2], ["1.0 Exp(10)"],
                                                 [("OK", None, "OK")]),
        "SpInterpSteps": lambda: spi.SpInterpSteps(),
        "interp_steps nrst": lambda: spi.interp_steps(
            x, y, z, x[:2], y[:2], ["1.0 Exp(10)"], [("OK", None, "OK")], neb_sel_mthd="nrst",
            n_nebs=2),
        "SpInterpNeighborGrouping": lambda: nebs.SpInterpNeighborGrouping("nrst", 2, None, x, y),
        "OrdinaryKriging": lambda: spi.OrdinaryKriging(x, y, z[0], x, y,
                                                       model="1.0 Exp(1000)").krige(),
        "cells_in_polygons": lambda: driver.cells_in_polygons(x, y, [(x, y)]),
        "stats_table": lambda: driver.stats_table(z, {}, []),
        "interpolate_grid": lambda: driver.interpolate_grid(
            x, y, z, ["1.0 Exp(1000)"], [("OK", None, "OK")], cell_size=250.0),
        "fit_steps": lambda: fitvgs.fit_steps(x, y, z),
        "krige_loo": lambda: steps.krige_loo(x, y, z, ["1.0 Exp(1000)"]),
        "warm_fit_steps": lambda: warmstart.warm_fit_steps(x, y, z, None),
    }
    for name, fn in calls.items():
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            fn()


def test_noalloc_limits_match_header():
    txt = (ROOT / "include" / "spinterps_gb300.h").read_text()
    stns = int(re.search(r"#define SPI_NOALLOC_MAX_STNS (\d+)", txt).group(1))
    steps = int(re.search(r"#define SPI_NOALLOC_MAX_STEPS (\d+)", txt).group(1))
    assert (stns, steps) == (nat.SPI_NOALLOC_MAX_STNS, nat.SPI_NOALLOC_MAX_STEPS)


def test_entry_points_check_arguments_before_any_gpu_work():
    """Invalid arguments come back as status codes (no GPU is touched): the
    per-cell neighbourhood kernel, the single-neighbourhood classes, the
    driver-flow kernels, the double-float variance, the tier decision and
    the FMA-rate kernel."""
    lib = nat.load()
    c_i64 = ctypes.c_int64
    dom = nat.DomainT()
    out = nat.OutT()
    vg = nat.VgT()
    vg.n_comp = 1
    dummy = ctypes.c_void_p(8)  # never dereferenced on these paths
    ARG, TOO_LARGE, VG = 1, 5, 2
    assert lib.spi_local_cells(None, 0, 8, None, 1, None, None, None, 0, None, None, 0.0, 2.0,
                               0, None, None, None) == ARG
    assert lib.spi_local_cells(ctypes.byref(dom), 0, 65, dummy, 1, dummy, dummy, dummy, 1,
                               dummy, dummy, 0.0, 2.0, 0, ctypes.byref(out), dummy,
                               None) == TOO_LARGE
    assert lib.spi_local_cells(ctypes.byref(dom), 7, 8, dummy, 1, dummy, dummy, dummy, 1, dummy,
                               dummy, 0.0, 2.0, 0, ctypes.byref(out), dummy, None) == ARG
    # spi_local_groups: argument checks that return before any CUDA call
    grp_args = lambda kind, k, scratch, nbytes: (  # noqa: E731
        ctypes.byref(dom), kind, k, dummy, 4, dummy, None, 1, dummy, dummy, dummy, 1, dummy,
        dummy, 0.0, 0, ctypes.byref(out), scratch, nbytes, dummy, None)
    dom.n_cells = 10
    out.est = dummy
    for f in ("cell_x", "cell_y", "stn_x", "stn_y"):
        setattr(dom, f, dummy)
    assert lib.spi_local_groups(None, *grp_args(0, 8, dummy, 1 << 30)[1:]) == ARG
    assert lib.spi_local_groups(*grp_args(3, 8, dummy, 1 << 30)) == ARG  # IDW: per cell
    assert lib.spi_local_groups(*grp_args(0, 65, dummy, 1 << 30)) == TOO_LARGE
    aligned = ctypes.c_void_p(64)
    assert lib.spi_local_groups(*grp_args(0, 8, ctypes.c_void_p(72), 1 << 30)) == ARG
    need = lib.spi_local_groups_scratch_bytes(0, 8, 0, 4, 1)
    assert lib.spi_local_groups(*grp_args(0, 8, aligned, need - 1)) == TOO_LARGE
    # scratch: the pinv check's slots, then per (group, step) the inverse and its status
    mm = 9
    pinv = (152 * 2 * mm * mm * 8 + 15) // 16 * 16
    assert need == pinv + 4 * (mm * mm * 8 + 4)
    assert lib.spi_local_groups_scratch_bytes(2, 16, 3, 100, 7) == (
        (152 * 2 * 20 * 20 * 8 + 15) // 16 * 16 + 700 * (20 * 20 * 8 + 4))
    assert lib.spi_local_groups_scratch_bytes(1, 16, 3, 100, 7) == (
        (152 * 2 * 16 * 16 * 8 + 15) // 16 * 16 + 700 * (16 * 16 * 8 + 4))
    assert lib.spi_local_groups_scratch_bytes(4, 16, 0, 1, 1) == -1
    dom.n_cells = 0
    out.est = None
    for f in ("cell_x", "cell_y", "stn_x", "stn_y"):
        setattr(dom, f, None)
    assert lib.spi_legacy_system(9, dummy, dummy, 5, None, 0, ctypes.byref(vg), dummy, dummy,
                                 dummy, dummy, None, None) == ARG
    vg0 = nat.VgT()
    assert lib.spi_legacy_system(0, dummy, dummy, 5, None, 0, ctypes.byref(vg0), dummy, dummy,
                                 dummy, dummy, None, None) == VG
    assert lib.spi_legacy_points(0, dummy, dummy, dummy, None, 5, dummy, dummy, None, -1, 0,
                                 ctypes.byref(vg), dummy, dummy, dummy, dummy, dummy, None,
                                 None, None) == ARG
    assert lib.spi_points_in_polygons(dummy, dummy, -1, 0, None, None, None, None, dummy,
                                      None) == ARG
    assert lib.spi_points_in_polygons(dummy, dummy, 0, 0, None, None, None, None, dummy,
                                      None) == 0
    assert lib.spi_field_stats(dummy, 0, -1, 10, 10, 0, dummy, 10, dummy, None) == ARG
    assert lib.spi_field_stats(dummy, 0, 70000, 10, 10, 0, dummy, 10, dummy, None) == TOO_LARGE
    assert lib.spi_round_fields(dummy, 0, -1, 3, None) == ARG
    assert lib.spi_round_fields(dummy, 0, 10, 400, None) == ARG
    assert lib.spi_round_fields(dummy, 0, 0, 3, None) == 0
    assert lib.spi_krige_var_df(None, None, None, 1e10, None) == ARG
    assert lib.spi_krige_tier(None, None, 0, None, None, None, None, None, 0.0, 0.0, 0.0, 0.0,
                              None, None, None, None) == ARG
    assert lib.spi_peak_fma(1, 0, dummy, ctypes.byref(c_i64()), None) == ARG


def test_interp_args_match_the_oracle():
    """The product's interpolation tuples (interp/prepare.py:638-695) equal
    the oracle's for every method mix."""
    from spinterps_gb300.steps import interp_args_for
    for methods in (["OK"], ["OK", "SK", ("IDW", 2.0), ("IDW", 1.0), "NNB"], ["EDK"]):
        for ev in (False, True):
            assert interp_args_for(methods, est_vars=ev) == port.interp_args_for(methods, ev)


# Tokens the reference's string rules meet in float(): Python accepts
# surrounding whitespace, digit-group underscores, inf / infinity / nan in
# any case; it rejects hexadecimal, 'nan(...)', a lone '.', empty tokens.
_SILLS = ["1", "0.5", ".5", "5.", "1e3", "1E-3", "-0.2", "+0.2", "inf", "-inf", "nan", "NaN",
          "Infinity", "1_0", "1__0", "_1", "1_", "0x10", "1.5e", "", "1.0\t", "\t1.0", "1d3",
          "1e400", "1e-400", "1.0.0", "1.5_0", "1e1_0"]
_NAMES = ["Nug", "Sph", "Exp", "Lin", "Gau", "Pow", "Hol", "Rng", "Foo", "exp", ""]
_RANGES = ["0", "10", "1e5", "-5", "1e-9", " 5", "\t5", "5\t", "1_000", "inf", "nan", "",
           "1e+5", "3)x", "3))", "(3", "0x1p3", "nan(1)"]


def _fuzz_strings(n, seed):
    import random
    rng = random.Random(seed)
    for _ in range(n):
        comps = []
        for _ in range(rng.choice([1, 1, 2, 2, 3, 4, 5])):
            comps.append(rng.choice(["", " ", "\t"]) + rng.choice(_SILLS) +
                         rng.choice([" ", "  ", "\t", ""]) + rng.choice(_NAMES) + "(" +
                         rng.choice(_RANGES) + rng.choice([")", ")", ")x", ""]))
        s = comps[0]
        for c in comps[1:]:
            s += rng.choice(["+", " + ", "+ ", " +", "++"]) + c
        yield s


def _same(a, b):
    return a == b or (np.isnan(a) and np.isnan(b))


def test_parse_vg_fuzz_matches_reference_rules():
    """spi_parse_vg against the oracle's restatement of
    cyth/interpmthds.pyx:174-184 on seeded random strings: the same
    components, or an error where the reference raises."""
    for s in _fuzz_strings(6000, 7):
        try:
            ref = port.parse_vg_str(s)
        except (ValueError, KeyError):
            ref = None
        rc, v = _parse(s)
        if len(s.encode().split(b"+")) > 4:
            assert rc == 5, s  # at most 4 components, checked before the parse
        elif ref is None:
            assert rc == 2, s
        else:
            assert rc == 0 and v.n_comp == len(ref), s
            for k, (code, sill, rng) in enumerate(ref):
                assert v.code[k] == code and _same(v.sill[k], sill) and v.range[k] == rng, s


def test_nuggetness_fuzz_matches_reference_rules():
    """spi_check_full_nuggetness against the oracle's restatement of
    misc.py:1074-1105 on the same kind of strings."""
    for s in _fuzz_strings(3000, 11):
        for mvv in (0.0, 1e-4):
            try:
                ref = port.check_full_nuggetness(s, mvv)
            except (ValueError, IndexError):
                ref = None
            out = nat.c_i32(-1)
            rc = nat.lib().spi_check_full_nuggetness(s.encode(), mvv, ctypes.byref(out))
            if ref is None:
                assert rc == 2, s
            else:
                assert rc == 0 and bool(out.value) == bool(ref), (s, mvv)
