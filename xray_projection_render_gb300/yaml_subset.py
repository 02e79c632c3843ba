"""A reader for the subset of YAML the reference's scene and deformation files
use (examples/*.yaml): block mappings and sequences (a sequence may sit at
its key's indentation), flow sequences and mappings on one line, comments,
plain and quoted scalars.  The reference decodes these files with
gopkg.in/yaml.v3 (main.go:63-76, 97-110); anchors, tags, multi-line flow
collections and block scalars are outside the subset and raise ValueError.

Numbers keep their YAML type (int or float); the engine's schema reader
takes either where the reference takes a float64.
"""
from __future__ import annotations

import json
import re

_INT = re.compile(r"^[-+]?(0|[1-9][0-9]*)$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")


def _strip_comment(line: str) -> str:
    q = None
    for k, c in enumerate(line):
        if q:
            if c == q:
                q = None
        elif c in "'\"":
            q = c
        elif c == "#" and (k == 0 or line[k - 1] in " \t"):
            return line[:k]
    return line


def _split_flow(text: str) -> list:
    """Top-level comma-separated parts of a flow collection's inside."""
    parts, depth, q, cur = [], 0, None, []
    for c in text:
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
        elif c == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
            continue
        cur.append(c)
    tail = "".join(cur).strip()
    if tail:
        parts.append(tail)
    return parts


def _key_split(text: str):
    """(key, rest) for `key: rest` / `key:`, or None when `text` is no mapping entry."""
    q, depth = None, 0
    for k, c in enumerate(text):
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
        elif c == ":" and depth == 0 and (k + 1 == len(text) or text[k + 1] in " \t"):
            return _scalar(text[:k].strip()), text[k + 1:].strip()
    return None


def _scalar(text: str):
    t = text.strip()
    if t.startswith("[") or t.startswith("{"):
        close = "]" if t[0] == "[" else "}"
        if not t.endswith(close):
            raise ValueError(f"unsupported YAML (multi-line flow collection): {text!r}")
        inner = _split_flow(t[1:-1])
        if t[0] == "[":
            return [_scalar(p) for p in inner]
        out = {}
        for p in inner:
            kv = _key_split(p)
            if kv is None:
                raise ValueError(f"bad flow mapping entry {p!r}")
            out[kv[0]] = _scalar(kv[1]) if kv[1] else None
        return out
    if len(t) >= 2 and t[0] == t[-1] == '"':
        return json.loads(t)
    if len(t) >= 2 and t[0] == t[-1] == "'":
        return t[1:-1].replace("''", "'")
    if t in ("", "~", "null", "Null", "NULL"):
        return None
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        return float(t)
    if t[0] in "&*!|>":
        raise ValueError(f"unsupported YAML construct: {text!r}")
    return t


class _Parser:
    def __init__(self, text: str):
        self.lines = []
        for raw in text.splitlines():
            if raw.strip() in ("---", "..."):
                continue
            s = _strip_comment(raw).rstrip()
            if not s.strip():
                continue
            if "\t" in s[: len(s) - len(s.lstrip())]:
                raise ValueError("tabs in YAML indentation")
            self.lines.append([len(s) - len(s.lstrip(" ")), s.strip()])

    def block(self, i: int, indent: int):
        if i >= len(self.lines):
            return None, i
        ind, content = self.lines[i]
        if content == "-" or content.startswith("- "):
            return self.sequence(i, ind)
        if _key_split(content) is not None:
            return self.mapping(i, ind)
        return _scalar(content), i + 1

    def sequence(self, i: int, indent: int):
        out = []
        while i < len(self.lines):
            ind, content = self.lines[i]
            if ind != indent or not (content == "-" or content.startswith("- ")):
                break
            item = content[1:].strip()
            if not item:
                if i + 1 < len(self.lines) and self.lines[i + 1][0] > indent:
                    v, i = self.block(i + 1, self.lines[i + 1][0])
                else:
                    v, i = None, i + 1
            elif _key_split(item) is not None and item[0] not in "[{'\"":
                # `- key: value` opens a mapping at the key's column
                col = indent + (len(content) - len(item))
                self.lines[i] = [col, item]
                v, i = self.mapping(i, col)
            elif item == "-" or item.startswith("- "):
                col = indent + (len(content) - len(item))
                self.lines[i] = [col, item]
                v, i = self.sequence(i, col)
            else:
                v, i = _scalar(item), i + 1
            out.append(v)
        return out, i

    def mapping(self, i: int, indent: int):
        out = {}
        while i < len(self.lines):
            ind, content = self.lines[i]
            if ind != indent or content == "-" or content.startswith("- "):
                break
            kv = _key_split(content)
            if kv is None:
                raise ValueError(f"expected `key: value`, got {content!r}")
            key, rest = kv
            if rest:
                out[key] = _scalar(rest)
                i += 1
                continue
            i += 1
            if i < len(self.lines) and self.lines[i][0] > indent:
                out[key], i = self.block(i, self.lines[i][0])
            elif (i < len(self.lines) and self.lines[i][0] == indent
                  and (self.lines[i][1] == "-" or self.lines[i][1].startswith("- "))):
                out[key], i = self.sequence(i, indent)
            else:
                out[key] = None
        return out, i


def loads(text: str):
    """The document in `text` as dicts, lists and scalars."""
    p = _Parser(text)
    if not p.lines:
        return None
    v, i = p.block(0, p.lines[0][0])
    if i != len(p.lines):
        raise ValueError(f"unexpected YAML content at {p.lines[i][1]!r}")
    return v


__all__ = ["loads"]
