"""CPU restatement of the reference's collection text reader.

TEST INFRASTRUCTURE ONLY (the checker of hyset_collection_parse).

read_text follows hyset::collection::read_collection
(include/hyset/collection.hpp:93-177) and split (collection.hpp:16-24):
  * lines come from std::getline on '\\n'; the loop `while (!eof)` also yields
    the text after the last '\\n' (nothing when the text ends with '\\n');
  * empty lines are skipped (line.empty());
  * a line is split by std::getline(ss, item, ' '): every ' ' ends an item,
    so two spaces or a leading space give an empty item, while a space at
    the very end of the line gives no further item;
  * each item becomes atoi(item) cast to unsigned: leading white space
    (' ', '\\t', '\\n', '\\v', '\\f', '\\r') is skipped, an optional sign, then
    decimal digits up to the first other byte; no digits give 0.
Pure Python, for small inputs.
"""
from __future__ import annotations

import numpy as np

_SPACE = b" \t\n\v\f\r"


def _atoi(item: bytes) -> int:
    i = 0
    while i < len(item) and item[i] in _SPACE:
        i += 1
    sign = 1
    if i < len(item) and item[i] in b"+-":
        sign = -1 if item[i] == ord("-") else 1
        i += 1
    v = 0
    while i < len(item) and 48 <= item[i] <= 57:
        v = v * 10 + item[i] - 48
        i += 1
    return (sign * v) & 0xFFFFFFFF


def _split(line: bytes) -> list:
    items, cur, i = [], bytearray(), 0
    while i < len(line):
        if line[i] == 32:
            items.append(bytes(cur))
            cur = bytearray()
        else:
            cur.append(line[i])
        i += 1
    if cur:  # text after the last delimiter; none when the line ends with ' '
        items.append(bytes(cur))
    return items


def read_text(data: bytes):
    """(tokens uint32[T], sizes uint32[n], empty_items) of the text as the
    reference reads it; empty_items counts items that were empty or had no
    digits (atoi gives 0 for them)."""
    toks, sizes, empty = [], [], 0
    lines = data.split(b"\n")
    if lines and lines[-1] == b"":
        lines = lines[:-1]
    for line in lines:
        if not line:
            continue
        items = _split(line)
        for it in items:
            stripped = it.strip(_SPACE).lstrip(b"+-")
            if not stripped[:1].isdigit():
                empty += 1
            toks.append(_atoi(it))
        sizes.append(len(items))
    return np.array(toks, dtype=np.uint32), np.array(sizes, dtype=np.uint32), empty


def write_text(tokens, starts, sizes, crlf: bool = False) -> bytes:
    """The reference's format: one set per line, tokens split by one space."""
    end = "\r\n" if crlf else "\n"
    out = []
    for s, z in zip(starts, sizes):
        out.append(" ".join(str(int(t)) for t in tokens[int(s):int(s) + int(z)]) + end)
    return "".join(out).encode()
