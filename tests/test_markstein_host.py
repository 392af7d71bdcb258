"""The operand windows of the bit-faithful FP64 policy's division through a
reciprocal (Markstein's correction of RN(a * RN(1/b))), checked on the host
with its correctly rounded fma: bit-identical to RN(a/b) on 2 * 10^7 operand
pairs inside the windows, including signed zero numerators; not so for
subnormal numerators, which therefore take the IEEE division on the device."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_markstein_windows(tmp_path):
    exe = str(tmp_path / "markstein_host")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "markstein_host.c"),
                           "-o", exe, "-lm"])
    inside, outside = map(int, subprocess.check_output([exe, "10000000"], text=True).split())
    assert inside == 0
    assert outside > 0


def test_quotient_integer_rounding_step(tmp_path):
    """The division's last rounding step on the integer pipe (the choice
    between RN(x * RN(1/c)) and its neighbours from the sign and size of the
    exact remainder), with the device's integer steps on the host: identical
    to RN(x/c) wherever it applies, on 3 * 10^7 cases that include
    quotients next to a midpoint and within a few ulps of a power of two,
    and on subnormal and tiny numerators scaled into the window."""
    exe = str(tmp_path / "quotient_host")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "quotient_host.c"),
                           "-o", exe, "-lm"])
    bad, applied, skipped, tiny_bad, tiny = map(int, subprocess.check_output([exe, "3000000"], text=True).split())
    assert bad == 0
    # numerators below the window whose quotient is normal, scaled by 2^256
    # on the integer pipe
    assert tiny_bad == 0 and tiny > 10**6
    # it applies to most cases; quotients at powers of two and exact
    # quotients with a short significand (a zero low word) take the FMA
    assert applied > 3 * skipped > 0


def test_one_minus_integer_pipe(tmp_path):
    """1 - x for x in [0.5, 2) on the integer pipe (exact by Sterbenz's
    lemma), with the device's integer steps on the host: identical to the
    IEEE subtraction on 1.2 * 10^7 values of the window, its ends and their
    neighbours; the window test refuses exactly the values outside it."""
    exe = str(tmp_path / "one_minus_host")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "one_minus_host.c"),
                           "-o", exe])
    bad, cases, outside = map(int, subprocess.check_output([exe, "3000000"], text=True).split())
    assert bad == 0
    assert cases > 10**7 and outside > 10**6


def test_subnormal_quotient_integer_grid(tmp_path):
    """Quotients below 2^-1021 by a grid-independent constant, rounded on the
    integer grid of the subnormals (N = RN(X/c) for X = |x| * 2^1074: below
    2^51 from RN(X * RN(1/c)) rounded to an integer and the exact remainder,
    from 2^51 from that product's own remainder and fraction), with the
    device's steps on the host: identical to RN(x/c) on about 1.5 * 10^7
    cases, exact ties (also at the top of the range) and exact quotients
    included."""
    exe = str(tmp_path / "subnormal_quotient_host")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off",
                           os.path.join(HERE, "native", "subnormal_quotient_host.c"), "-o", exe, "-lm"])
    bad, cases, upper = map(int, subprocess.check_output([exe, "2000000"], text=True).split())
    assert bad == 0
    assert cases > 10**7 and upper > 10**6


def test_division_forms_cover_the_range():
    """Which numerators the FP64 division by a grid-independent constant
    leaves to the IEEE division, exponent by exponent (the device's window,
    tiny and integer-grid tests of F64Exact::divu, restated): of the
    numerators of exponent at most 960 whose quotient's exponent is at most
    1000, none when the divisor lies in [2^-100, 2^40]; above 2^40, only
    those of exponent at least -960 whose quotient lies in
    [2^-1021, 2^-1000)."""
    def forms(ex, eff, ec):
        window = 63 <= ex <= 1983 and 0 <= ex - ec + 1000 <= 2000
        tiny = ex < 63 and eff + 1021 >= ec
        below = eff - ec <= -1022
        return window or tiny or below

    for ec in range(1023 - 100, 1023 + 101):
        for ex in range(0, 2047):
            for eff in (range(-51, 1) if ex == 0 else (ex,)):
                if ex > 1983 or ex - ec > 1000 or forms(ex, eff, ec):
                    continue
                assert ec - 1023 > 40, (ec - 1023, ex - 1023)
                assert ex - 1023 >= -960 and -1021 <= ex - ec <= -1001, (ec - 1023, ex - 1023)


def test_division_warp_forms(tmp_path):
    """The division by a grid-independent constant as a warp of 32 lanes
    takes it (the window; window or tiny numerators scaled by 2^256; those
    or quotients below 2^-1021 on the integer grid; else the IEEE
    division), with the device's steps on the host: every lane identical to
    RN(x/c) on 9.6 * 10^6 lanes of warps that mix the numerator classes,
    every form taken."""
    exe = str(tmp_path / "divu_warp_host")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", os.path.join(HERE, "native", "divu_warp_host.c"),
                           "-o", exe, "-lm"])
    bad, lanes, *forms = map(int, subprocess.check_output([exe, "300000"], text=True).split())
    assert bad == 0
    assert lanes == 300000 * 32
    assert all(f > 10000 for f in forms), forms
