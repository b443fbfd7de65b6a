"""Block-style YAML for big-wave's simulation directories: the metadata files a run writes
(detector_metadata.yaml, source_geometry.yaml, history_metadata.yaml) and the prepared
configuration it reads (config.yaml, computed.yaml, subconfig.yaml).

big-wave writes them with ruamel's round-trip dumper, mapping indent 2, sequence indent 4, dash
offset 2 (big-wave/config.py:516-520). Neither ruamel nor PyYAML is a dependency here, so this
module writes that layout for the value types the metadata holds (mappings, sequences, str,
int, float, bool, None) and reads the same subset back (YAML 1.2 core-schema scalars: null/~,
true/false, decimal ints, floats incl. .inf/.nan, single- and double-quoted strings, empty
flow collections and flow sequences of scalars; node tags such as !!python/tuple are skipped).
"""
from __future__ import annotations

import math
import re
from pathlib import Path
from typing import Any

_INT = re.compile(r"^[-+]?[0-9]+$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")
_SPECIAL = {".inf": math.inf, "+.inf": math.inf, "-.inf": -math.inf, ".nan": math.nan,
            ".Inf": math.inf, "-.Inf": -math.inf, ".NaN": math.nan, ".INF": math.inf, ".NAN": math.nan}
_RESERVED = {"null", "Null", "NULL", "~", "true", "True", "TRUE", "false", "False", "FALSE", ""}


# -- writing ------------------------------------------------------------------------------------
def _scalar(v: Any) -> str:
    if v is None:
        return ""
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int) or (hasattr(v, "dtype") and getattr(v.dtype, "kind", "") in "iu"):
        return str(int(v))
    if isinstance(v, float) or (hasattr(v, "dtype") and getattr(v.dtype, "kind", "") == "f"):
        f = float(v)
        if math.isnan(f):
            return ".nan"
        if math.isinf(f):
            return ".inf" if f > 0 else "-.inf"
        return repr(f)
    s = str(v)
    if any(not _printable(c) for c in s):
        return _double_quoted(s)
    if (s in _RESERVED or s in _SPECIAL or _INT.match(s) or _FLOAT.match(s) or s != s.strip()
            or any(c in s for c in ":#{}[],&*!|>'\"%@`") or s.startswith(("-", "?"))):
        return "'" + s.replace("'", "''") + "'"
    return s


def _printable(c: str) -> bool:
    """YAML's printable set (YAML 1.2, section 5.1) minus the line breaks."""
    o = ord(c)
    return (0x20 <= o <= 0x7E or 0xA0 <= o <= 0xD7FF or 0xE000 <= o <= 0xFFFD
            or 0x10000 <= o <= 0x10FFFF) and o not in (0x2028, 0x2029, 0xFEFF)


_ESC_OUT = {"\\": "\\\\", '"': '\\"', "\n": "\\n", "\t": "\\t", "\r": "\\r", "\0": "\\0"}


def _double_quoted(s: str) -> str:
    out = []
    for c in s:
        if c in _ESC_OUT:
            out.append(_ESC_OUT[c])
        elif _printable(c):
            out.append(c)
        elif ord(c) <= 0xFF:
            out.append(f"\\x{ord(c):02x}")
        elif ord(c) <= 0xFFFF:
            out.append(f"\\u{ord(c):04x}")
        else:
            out.append(f"\\U{ord(c):08x}")
    return '"' + "".join(out) + '"'


def _emit(v: Any, indent: int, out: list[str]) -> None:
    pad = " " * indent
    if isinstance(v, dict):
        for k, item in v.items():
            key = _scalar(k)
            if isinstance(item, dict) and item:
                out.append(f"{pad}{key}:")
                _emit(item, indent + 2, out)
            elif isinstance(item, (list, tuple)) and len(item) > 0:
                out.append(f"{pad}{key}:")
                _emit(list(item), indent + 2, out)
            elif isinstance(item, dict):
                out.append(f"{pad}{key}: {{}}")
            elif isinstance(item, (list, tuple)):
                out.append(f"{pad}{key}: []")
            else:
                s = _scalar(item)
                out.append(f"{pad}{key}:" + (f" {s}" if s else ""))
    elif isinstance(v, list):
        for item in v:
            if isinstance(item, dict) and item:
                sub: list[str] = []
                _emit(item, indent + 2, sub)
                out.append(f"{pad}- {sub[0].lstrip()}")
                out.extend(sub[1:])
            elif isinstance(item, (list, tuple)) and len(item) > 0:
                sub = []
                _emit(list(item), indent + 2, sub)
                out.append(f"{pad}- {sub[0].lstrip()}")
                out.extend(sub[1:])
            elif isinstance(item, dict):
                out.append(f"{pad}- {{}}")
            elif isinstance(item, (list, tuple)):
                out.append(f"{pad}- []")
            else:
                s = _scalar(item)
                out.append(f"{pad}-" + (f" {s}" if s else ""))
    else:
        out.append(pad + _scalar(v))


def dumps(obj: Any) -> str:
    out: list[str] = []
    _emit(obj, 0, out)
    return "\n".join(out) + "\n"


def save(path: Path | str, obj: Any) -> None:
    """Write `obj` to `path` (config.save's layout, big-wave/config.py:516-520)."""
    Path(path).write_text(dumps(obj), encoding="utf-8")


# -- reading ------------------------------------------------------------------------------------
def _parse_scalar(s: str) -> Any:
    s = s.strip()
    if s.startswith("'"):
        if not s.endswith("'") or len(s) < 2:
            raise ValueError(f"unterminated quoted scalar {s!r}")
        return s[1:-1].replace("''", "'")
    if s.startswith('"'):
        if not s.endswith('"') or len(s) < 2 or _quote_end(s, 0) != len(s) - 1:
            raise ValueError(f"unterminated quoted scalar {s!r}")
        return _unescape(s[1:-1])
    s = _strip_tag(s)
    if s in ("", "~", "null", "Null", "NULL"):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if s in _SPECIAL:
        return _SPECIAL[s]
    if _INT.match(s):
        return int(s)
    if _FLOAT.match(s):
        return float(s)
    if s == "[]":
        return []
    if s == "{}":
        return {}
    if s.startswith("[") and s.endswith("]"):
        return [_parse_scalar(p) for p in s[1:-1].split(",")]
    return s


_ESC_IN = {"0": "\0", "a": "\a", "b": "\b", "t": "\t", "\t": "\t", "n": "\n", "v": "\v", "f": "\f",
           "r": "\r", "e": "\x1b", " ": " ", '"': '"', "/": "/", "\\": "\\", "N": "\x85", "_": "\xa0",
           "L": "\u2028", "P": "\u2029"}


def _unescape(body: str) -> str:
    """The escapes of a double-quoted YAML scalar (YAML 1.2, section 5.7)."""
    out = []
    i = 0
    while i < len(body):
        c = body[i]
        if c != "\\":
            out.append(c)
            i += 1
            continue
        if i + 1 >= len(body):
            raise ValueError(f"dangling escape in {body!r}")
        e = body[i + 1]
        width = {"x": 2, "u": 4, "U": 8}.get(e)
        if width:
            digits = body[i + 2:i + 2 + width]
            if len(digits) != width or any(d not in "0123456789abcdefABCDEF" for d in digits):
                raise ValueError(f"bad escape in {body!r}")
            out.append(chr(int(digits, 16)))
            i += 2 + width
        elif e in _ESC_IN:
            out.append(_ESC_IN[e])
            i += 2
        else:
            raise ValueError(f"unknown escape \\{e} in {body!r}")
    return "".join(out)


def _quote_end(text: str, start: int) -> int:
    """Index of the quote closing the quoted scalar opening at text[start], or -1: a single-quoted
    scalar escapes its quote by doubling it, a double-quoted one by a backslash."""
    q = text[start]
    j = start + 1
    while j < len(text):
        c = text[j]
        if q == '"' and c == "\\":
            j += 2
            continue
        if c == q:
            if q == "'" and j + 1 < len(text) and text[j + 1] == "'":
                j += 2
                continue
            return j
        j += 1
    return -1


def _strip_comment(line: str) -> str:
    i = 0
    while i < len(line):
        c = line[i]
        if c in "'\"" and (i == 0 or line[i - 1] in " \t:-[{,"):
            end = _quote_end(line, i)
            if end < 0:
                return line.rstrip()
            i = end + 1
            continue
        if c == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i].rstrip()
        i += 1
    return line.rstrip()


def _strip_tag(text: str) -> str:
    """Drop a leading node tag (!!python/tuple, !!float, ...): the values are read by their text."""
    if text.startswith("!"):
        parts = text.split(None, 1)
        return parts[1] if len(parts) > 1 else ""
    return text


def _split_key(text: str):
    """'key: value' -> (key, value) honouring a quoted key; None if text is not a mapping entry."""
    if text.startswith(("'", '"')):
        j = _quote_end(text, 0)
        if j < 0:
            return None
        rest = text[j + 1:]
        if rest.startswith(":") and (len(rest) == 1 or rest[1] == " "):
            return _parse_scalar(text[:j + 1]), rest[1:].strip()
        return None
    m = re.match(r"^([^:#]+?):(\s|$)(.*)$", text)
    if not m:
        return None
    return _parse_scalar(m.group(1)), _strip_tag(m.group(3).strip())


def loads(text: str) -> Any:
    lines = []
    # only \n (and \r\n) break lines: str.splitlines would also split at control characters
    for raw in text.replace("\r\n", "\n").split("\n"):
        if raw.strip() in ("---", "...") or not raw.strip() or raw.lstrip().startswith("#"):
            continue
        line = _strip_comment(raw)
        if line.strip():
            lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    pos = 0

    def block(indent: int) -> Any:
        nonlocal pos
        if pos >= len(lines):
            return None
        ind, txt = lines[pos]
        if txt.startswith("- ") or txt == "-":
            seq = []
            while pos < len(lines) and lines[pos][0] == ind and (lines[pos][1].startswith("- ") or lines[pos][1] == "-"):
                item = _strip_tag(lines[pos][1][1:].strip())
                if not item:
                    pos += 1
                    seq.append(block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > ind else None)
                elif item.startswith("- ") or item == "-" or _split_key(item) is not None:
                    # a sequence or mapping that starts on the dash line: re-read it at its own indent
                    lines[pos] = (ind + 2, item)
                    seq.append(block(ind + 2))
                else:
                    seq.append(_parse_scalar(item))
                    pos += 1
            return seq
        mapping = {}
        while pos < len(lines) and lines[pos][0] == ind:
            kv = _split_key(lines[pos][1])
            if kv is None:
                raise ValueError(f"cannot parse YAML line {lines[pos][1]!r}")
            key, value = kv
            pos += 1
            if value == "":
                if pos < len(lines) and (lines[pos][0] > ind or
                                         (lines[pos][0] == ind and lines[pos][1].startswith("- "))):
                    mapping[key] = block(lines[pos][0])
                else:
                    mapping[key] = None
            else:
                mapping[key] = _parse_scalar(value)
        return mapping

    if not lines:
        return None
    result = block(lines[0][0])
    if pos != len(lines):
        raise ValueError(f"unexpected indentation at YAML line {lines[pos][1]!r}")
    return result


def load(path: Path | str) -> Any:
    return loads(Path(path).read_text(encoding="utf-8"))
