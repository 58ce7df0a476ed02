"""The oracle's restatement of Context::flush (src/context.rs:50-92) against bytes written
out by hand from the reference's format strings.  CPU only."""
import numpy as np

from oracle import oracle as O


def cell(ch, r=0, g=0, b=0):
    return ord(ch) | (r << 8) | (g << 16) | (b << 24)


CELLS = np.array([cell("@", 255, 7, 10), cell("\n"), cell(" ")], np.uint32)


def test_plain_is_the_chars_and_println_newline():
    assert O.flush(CELLS, True, O.FLUSH_PLAIN) == b"@\n \n"
    # terminal contexts queue MoveTo(0,0) first
    assert O.flush(CELLS, False, O.FLUSH_PLAIN) == b"\x1b[1;1H@\n \n"


def test_ansi_is_crossterm_styled_content_per_cell():
    one = b"\x1b[48;2;25;25;25m\x1b[38;2;255;7;10m@\x1b[0m"
    nl = b"\x1b[48;2;25;25;25m\x1b[38;2;0;0;0m\n\x1b[0m"
    sp = b"\x1b[48;2;25;25;25m\x1b[38;2;0;0;0m \x1b[0m"
    assert O.flush(CELLS, True, O.FLUSH_ANSI) == one + nl + sp
    assert O.flush(CELLS, False, O.FLUSH_ANSI) == b"\x1b[1;1H" + one + nl + sp


def test_html_is_one_unclosed_span_per_cell():
    want = (b'<span style="color:rgb(255,7,10)">@' b'<span style="color:rgb(0,0,0)">\n'
            b'<span style="color:rgb(0,0,0)"> ')
    assert O.flush(CELLS, True, O.FLUSH_HTML) == want


def test_empty_frame_and_digit_widths():
    assert O.flush(np.zeros(0, np.uint32), True, O.FLUSH_PLAIN) == b"\n"
    assert O.flush(np.zeros(0, np.uint32), True, O.FLUSH_HTML) == b""
    c = np.array([cell(".", 9, 10, 100), cell("%", 99, 0, 255)], np.uint32)
    assert O.flush(c, True, O.FLUSH_HTML) == (b'<span style="color:rgb(9,10,100)">.'
                                              b'<span style="color:rgb(99,0,255)">%')
