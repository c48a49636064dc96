"""The slice runner's journal (the reference's run_range.sh contract): the
resume point is the end of the contiguous PASS chain from the range's start;
RETRY rows and PASS rows off the chain do not move it. Host logic only."""
import gbc


def write(path, rows):
    path.write_text("".join(r + "\n" for r in rows))


def test_resume_walks_the_pass_chain(tmp_path):
    j = tmp_path / "journal.txt"
    assert gbc.journal_resume(j, 1000) == 1000  # no journal yet
    write(j, [
        "PASS 1000 1998 2026-01-01T00:00:00Z version=x result=PASS release=r",
        "RETRY 2000 2998 2026-01-01T00:00:01Z reason=-3",
        "PASS 2000 2998 2026-01-01T00:00:02Z version=x result=PASS release=r attempts=2",
        "PASS 5000 5998 2026-01-01T00:00:03Z version=x result=PASS release=r",  # off the chain
        "garbage line",
    ])
    assert gbc.journal_resume(j, 1000) == 3000
    assert gbc.journal_resume(j, 5000) == 6000
    assert gbc.journal_resume(j, 4000) == 4000


def test_retry_rows_alone_do_not_advance(tmp_path):
    j = tmp_path / "journal.txt"
    write(j, ["RETRY 10 18 2026-01-01T00:00:00Z reason=-3"])
    assert gbc.journal_resume(j, 10) == 10
