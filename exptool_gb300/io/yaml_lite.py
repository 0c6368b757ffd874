"""A YAML subset reader for the component info strings of EXP snapshot files
(psp_io.py:138-139 and spl_io.py:134-136 of the reference parse them with
``yaml.safe_load``; PyYAML is not a dependency here).

Supported: block mappings (nested by indentation), block sequences (``- x``),
flow mappings ``{a: 1, b: [2, 3]}`` and flow sequences, ``#`` comments, and
plain or quoted scalars resolved by the YAML 1.1 type rules (integers in
decimal, octal, hex and binary, floats with a decimal point, .inf/.nan,
booleans, null, otherwise strings).  Anchors, tags, multi-line scalars and
multiple documents are not.
"""
from __future__ import annotations

import re

# plain-scalar resolution of the YAML 1.1 type repository (yaml.org/type/bool,
# int, float, null): e.g. "1e-3" (no dot) is a string, "010" is octal 8, "Yes"
# is true.  The one-letter y/n booleans of that repository are left as strings.
_BOOL_T = {"yes", "Yes", "YES", "true", "True", "TRUE", "on", "On", "ON"}
_BOOL_F = {"no", "No", "NO", "false", "False", "FALSE", "off", "Off", "OFF"}
_NULL = {"", "~", "null", "Null", "NULL"}
_INT_DEC = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_INT_OCT = re.compile(r"^[-+]?0[0-7_]+$")
_INT_HEX = re.compile(r"^[-+]?0x[0-9a-fA-F_]+$")
_INT_BIN = re.compile(r"^[-+]?0b[01_]+$")
_FLOAT = re.compile(r"^([-+]?[0-9][0-9_]*\.[0-9_]*([eE][-+][0-9]+)?|\.[0-9][0-9_]*([eE][-+][0-9]+)?)$")
_INF = re.compile(r"^[-+]?\.(inf|Inf|INF)$")
_NAN = re.compile(r"^\.(nan|NaN|NAN)$")


def scalar(tok: str):
    """Resolve one plain or quoted scalar token."""
    t = tok.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        body = t[1:-1]
        return body.replace("''", "'") if t[0] == "'" else bytes(body, "utf-8").decode("unicode_escape")
    if t in _NULL:
        return None
    if t in _BOOL_T:
        return True
    if t in _BOOL_F:
        return False
    u = t.replace("_", "")
    if _INT_DEC.match(t):
        return int(u)
    if _INT_HEX.match(t):
        return int(u, 16)
    if _INT_BIN.match(t):
        return int(u.replace("0b", "", 1), 2)
    if _INT_OCT.match(t):
        return int(u, 8)
    if _FLOAT.match(t):
        return float(u)
    if _INF.match(t):
        return float("-inf") if t.startswith("-") else float("inf")
    if _NAN.match(t):
        return float("nan")
    return t


def _strip_comment(line: str) -> str:
    out, q = [], None
    for i, c in enumerate(line):
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(c)
    return "".join(out).rstrip()


def _split_top(s: str, sep: str):
    """Split s at `sep` outside brackets and quotes."""
    parts, depth, q, cur = [], 0, None, []
    for c in s:
        if q:
            cur.append(c)
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        elif c in "[{":
            depth += 1
        elif c in "]}":
            depth -= 1
        if c == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(c)
    parts.append("".join(cur))
    return parts


def _key_value(s: str):
    """'key: value' -> (key, value) on the first top-level ': ' (or trailing ':')."""
    depth, q = 0, None
    for i, c in enumerate(s):
        if q:
            if c == q:
                q = None
            continue
        if c in "'\"":
            q = c
        elif c in "[{":
            depth += 1
        elif c in "]}":
            depth -= 1
        elif c == ":" and depth == 0 and (i + 1 == len(s) or s[i + 1] in " \t"):
            return s[:i].strip(), s[i + 1:].strip()
    return None


def flow(s: str):
    """A flow collection or a scalar."""
    s = s.strip()
    if s.startswith("{") and s.endswith("}"):
        out = {}
        inner = s[1:-1].strip()
        if inner:
            for item in _split_top(inner, ","):
                if not item.strip():
                    continue
                kv = _key_value(item.strip())
                if kv is None:
                    out[scalar(item)] = None
                else:
                    out[scalar(kv[0])] = flow(kv[1])
        return out
    if s.startswith("[") and s.endswith("]"):
        inner = s[1:-1].strip()
        return [flow(x) for x in _split_top(inner, ",")] if inner else []
    return scalar(s)


def load(text: str):
    """Parse one YAML document of the supported subset."""
    if isinstance(text, bytes):
        text = text.decode()
    lines = []
    for raw in text.replace("\t", "  ").splitlines():
        if raw.strip() in ("---", "..."):
            continue
        line = _strip_comment(raw)
        if line.strip():
            lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    if not lines:
        return None
    value, pos = _block(lines, 0, lines[0][0])
    if pos != len(lines):
        raise ValueError(f"unparsed YAML from line {pos}: {lines[pos][1]!r}")
    return value


def _block(lines, pos, indent):
    """Parse the block starting at lines[pos] with this indentation."""
    if lines[pos][1].startswith("- ") or lines[pos][1] == "-":
        out = []
        while pos < len(lines) and lines[pos][0] == indent and (lines[pos][1].startswith("- ") or
                                                                 lines[pos][1] == "-"):
            rest = lines[pos][1][1:].strip()
            pos += 1
            if not rest:
                if pos < len(lines) and lines[pos][0] > indent:
                    v, pos = _block(lines, pos, lines[pos][0])
                else:
                    v = None
                out.append(v)
            elif _key_value(rest) is not None and not rest.startswith(("{", "[")):
                # "- key: value" opens a mapping at the item's indentation
                sub = [(indent + 2, rest)]
                while pos < len(lines) and lines[pos][0] > indent:
                    sub.append(lines[pos])
                    pos += 1
                v, _ = _block(sub, 0, indent + 2)
                out.append(v)
            else:
                out.append(flow(rest))
        return out, pos
    if _key_value(lines[pos][1]) is None:
        return flow(lines[pos][1]), pos + 1
    out = {}
    while pos < len(lines) and lines[pos][0] == indent:
        kv = _key_value(lines[pos][1])
        if kv is None:
            raise ValueError(f"expected 'key: value', got {lines[pos][1]!r}")
        k, v = kv
        pos += 1
        if v == "":
            if pos < len(lines) and lines[pos][0] > indent:
                val, pos = _block(lines, pos, lines[pos][0])
            elif pos < len(lines) and lines[pos][0] == indent and lines[pos][1].startswith("- "):
                val, pos = _block(lines, pos, indent)       # sequence at the key's indentation
            else:
                val = None
        else:
            val = flow(v)
        out[scalar(k)] = val
    return out, pos
