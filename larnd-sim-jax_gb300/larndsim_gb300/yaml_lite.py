"""Minimal block-YAML reader for detector-property and pixel-layout files.

The reference loads its detector configuration with PyYAML
(src/larndsim/consts_jax.py:303-318).  PyYAML is not installed on the
machines this package targets, so this module reads the subset of YAML that
those files use: nested block mappings, block sequences (also at the same
indentation as their key), flow sequences ``[a, b, c]``, ``#`` comments and
int/float/bool/null/string scalars.  Anything outside that subset raises
``ValueError``.
"""

from __future__ import annotations

import re

_INT_RE = re.compile(r"^[-+]?\d+$")
_FLOAT_RE = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")


def _scalar(tok: str):
    tok = tok.strip()
    if tok == "" or tok in ("~", "null", "Null", "NULL"):
        return None
    if tok in ("true", "True", "TRUE"):
        return True
    if tok in ("false", "False", "FALSE"):
        return False
    if len(tok) >= 2 and tok[0] == tok[-1] and tok[0] in "'\"":
        return tok[1:-1]
    if _INT_RE.match(tok):
        return int(tok)
    if _FLOAT_RE.match(tok):
        return float(tok)
    if tok.startswith("["):
        return _flow_list(tok)
    return tok


def _flow_list(tok: str):
    tok = tok.strip()
    if not (tok.startswith("[") and tok.endswith("]")):
        raise ValueError(f"unsupported flow value: {tok!r}")
    inner = tok[1:-1]
    out, depth, cur = [], 0, ""
    for ch in inner:
        if ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(_scalar(cur))
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(_scalar(cur))
    return out


def _strip_comment(line: str) -> str:
    # The supported files never put '#' inside quoted strings.
    pos = line.find("#")
    return line if pos < 0 else line[:pos]


def _lines(text: str):
    out = []
    for raw in text.splitlines():
        body = _strip_comment(raw).rstrip()
        if not body.strip() or body.strip() == "---":
            continue
        indent = len(body) - len(body.lstrip(" "))
        out.append((indent, body.strip()))
    return out


def _split_key(content: str):
    # "key: value" or "key:"; keys in the supported files are plain tokens.
    if content.endswith(":"):
        return content[:-1].strip(), ""
    pos = content.find(": ")
    if pos < 0:
        raise ValueError(f"expected 'key: value', got {content!r}")
    return content[:pos].strip(), content[pos + 2:].strip()


def _parse_block(lines, i, indent):
    if lines[i][1].startswith("- ") or lines[i][1] == "-":
        return _parse_list(lines, i, indent)
    return _parse_map(lines, i, indent)


def _parse_list(lines, i, indent):
    out = []
    while i < len(lines) and lines[i][0] == indent and (lines[i][1].startswith("- ") or lines[i][1] == "-"):
        item = lines[i][1][1:].strip()
        i += 1
        if item == "":
            if i < len(lines) and lines[i][0] > indent:
                val, i = _parse_block(lines, i, lines[i][0])
            else:
                val = None
            out.append(val)
        else:
            out.append(_scalar(item))
    return out, i


def _parse_map(lines, i, indent):
    out = {}
    while i < len(lines) and lines[i][0] == indent:
        content = lines[i][1]
        if content.startswith("- "):
            break
        key, rest = _split_key(content)
        key = _scalar(key)
        i += 1
        if rest != "":
            out[key] = _scalar(rest)
            continue
        if i < len(lines) and lines[i][0] > indent:
            val, i = _parse_block(lines, i, lines[i][0])
        elif i < len(lines) and lines[i][0] == indent and lines[i][1].startswith("- "):
            val, i = _parse_list(lines, i, indent)
        else:
            val = None
        out[key] = val
    return out, i


def loads(text: str):
    lines = _lines(text)
    if not lines:
        return None
    val, i = _parse_block(lines, 0, lines[0][0])
    if i != len(lines):
        raise ValueError(f"unparsed YAML content at line {i}: {lines[i]!r}")
    return val


def load(path: str):
    with open(path) as fh:
        return loads(fh.read())
