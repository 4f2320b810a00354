"""Restart-file naming and the info file's Fortran (100g15.5) text (igrid.F90:2719-2802)."""
from padeops_gb300.IncompressibleGrid import fortran_g15_5, restart_name


def test_restart_names():
    assert restart_name(1, "u", 300) == "RESTART_Run01_u.000300"
    assert restart_name(12, "info", 7) == "RESTART_Run12_info.000007"


def test_g15_5_matches_fortran_editing():
    cases = {0.0: "     0.0000    ", 0.123456: "    0.12346    ", 1.234567: "     1.2346    ",
             12.34567: "     12.346    ", 99999.4: "     99999.    ", 123456.7: "    0.12346E+06",
             0.0123456: "    0.12346E-01", -0.5: "   -0.50000    ", -2.5e-7: "   -0.25000E-06",
             9.999996: "     10.000    "}
    for x, want in cases.items():
        got = fortran_g15_5(x)
        assert got == want, (x, got, want)
        assert len(got) == 15
        assert abs(float(got) - x) <= 1e-4 * max(abs(x), 1e-30)
