"""The %d and %lf conversions of C's scanf family, for reading the reference's
input files (parameter files, rudy graphs) exactly as its fscanf / sscanf calls
do: leading white space is skipped, the longest numeric prefix is taken, and a
conversion that finds no number fails (the caller sees None).

scan_int(text, pos) and scan_double(text, pos) return (value, position after
the number), or (None, pos) when the conversion fails.
"""
import re

_WS = re.compile(r"[ \t\n\v\f\r]*")
_INT = re.compile(r"[+-]?[0-9]+")
_DEC = re.compile(r"[+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?")
_HEX = re.compile(r"[+-]?0[xX](?:[0-9a-fA-F]+\.?[0-9a-fA-F]*|\.[0-9a-fA-F]+)(?:[pP][+-]?[0-9]+)?")
_SPECIAL = re.compile(r"[+-]?(?:inf(?:inity)?|nan)", re.I)


def skip_space(text, pos):
    return _WS.match(text, pos).end()


def scan_int(text, pos=0):
    """%d: optional sign and at least one decimal digit."""
    p = skip_space(text, pos)
    m = _INT.match(text, p)
    if not m:
        return None, pos
    return int(m.group(0)), m.end()


def scan_double(text, pos=0):
    """%lf: a decimal or hexadecimal floating-point number, inf or nan."""
    p = skip_space(text, pos)
    for rx, conv in ((_HEX, float.fromhex), (_SPECIAL, float), (_DEC, float)):
        m = rx.match(text, p)
        if m:
            return conv(m.group(0)), m.end()
    return None, pos
