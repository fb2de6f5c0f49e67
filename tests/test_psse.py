"""The PSS/E v33 reader (psse.read_raw / read_dyr) on text written back from
the golden fixtures' tokenised records: every example case of the
reference round-trips to the same tokens, transformer records spanning
four lines and dynamic records spanning several lines included, and the
power systems built from the re-read records equal those built from the
fixtures.
"""
import numpy as np
import pytest

from helpers import psse

_SECTION_END = ["END OF BUS DATA, BEGIN LOAD DATA", "END OF LOAD DATA, BEGIN FIXED SHUNT DATA",
                "END OF FIXED SHUNT DATA, BEGIN GENERATOR DATA", "END OF GENERATOR DATA, BEGIN BRANCH DATA",
                "END OF BRANCH DATA, BEGIN TRANSFORMER DATA", "END OF TRANSFORMER DATA"]


def _raw_text(rec):
    lines = ["0, %r, 33, 0, 1, 60.00     / written by the round-trip test" % rec["baseMVA"],
             "first title line", "second title line"]
    for sec, end in zip(psse._SECTIONS, _SECTION_END):
        for r in rec[sec]:
            if sec == "transformer":
                lines += [", ".join(part) for part in r]
            else:
                lines.append(", ".join(r))
        lines.append("0 / " + end)
    return "\n".join(lines) + "\nQ\n"


def _dyr_text(records):
    # the model name and ident on the first line, then at most five
    # parameters a line, the closing '/' on the last one
    lines = []
    for tok in records:
        body = tok[:-1]
        lines.append("  ".join(body[:3]))
        rest = body[3:]
        for i in range(0, len(rest), 5):
            lines.append("      " + "  ".join(rest[i:i + 5]))
        lines[-1] += "  /"
        lines.append("")
    return "\n".join(lines)


@pytest.mark.parametrize("name", ["2bus.raw", "IEEE39.raw", "ieee9_v33.raw", "testdata/2bus.raw"])
def test_raw_round_trip(golden_cases, name):
    rec = golden_cases["raw"][name]
    back = psse.read_raw(_raw_text(rec))
    assert back["baseMVA"] == rec["baseMVA"]
    for sec in psse._SECTIONS:
        assert back[sec] == rec[sec], sec
    # the same power system either way
    a, b = psse.ps_from_records(rec), psse.ps_from_records(back)
    assert [(x.i, x.type, x.v0m, x.v0a) for x in a.buses] == [(x.i, x.type, x.v0m, x.v0a) for x in b.buses]
    assert [(x.fr, x.to, x.r, x.x, x.sh, x.tap, x.shift) for x in a.branches] == \
        [(x.fr, x.to, x.r, x.x, x.sh, x.tap, x.shift) for x in b.branches]


def test_dyr_round_trip(golden_cases):
    assert golden_cases["dyr"]
    for name, records in golden_cases["dyr"].items():
        assert psse.read_dyr(_dyr_text(records)) == records, name


def test_dyr_comments_blank_lines_and_commas():
    """Comment and blank lines are skipped; a record's first line splits on
    commas when it has one, else on blanks, and its continuation lines on
    either (src/parse.jl:115-136)."""
    text = "\n".join([
        "// a comment line",
        "",
        "1, 'TGOV1', 1, 0.05, 0.5, 1.2",
        "   0.0, 2.0  1.0, 0.0 /",
        "2 'SEXS' 1 0.1 10.0 100.0 0.05 -5.0 5.0 /",
    ])
    recs = psse.read_dyr(text)
    assert recs == [["1", "'TGOV1'", "1", "0.05", "0.5", "1.2", "0.0", "2.0", "1.0", "0.0", "/"],
                    ["2", "'SEXS'", "1", "0.1", "10.0", "100.0", "0.05", "-5.0", "5.0", "/"]]
    tg = psse._device(recs[0])
    ex = psse._device(recs[1])
    assert tg is not None and ex is not None
    assert tg.is_governor and ex.is_exciter


def test_dyr_trailing_comma_gives_an_empty_token_as_the_reference_does():
    """A first line ending in a comma leaves an empty token before the
    continuation, as the reference's split does."""
    recs = psse.read_dyr("1, 'TGOV1', 1, 0.05,\n 0.5 /")
    assert recs == [["1", "'TGOV1'", "1", "0.05", "", "0.5", "/"]]
