"""Fortran namelist reader for model.namelist files.

Restates the subset of list-directed namelist input the reference uses:
``&group key=value, ... /`` groups (repeatable), ``!`` comments, strings in
single or double quotes, integers, reals with e/d exponents, logicals and
comma separated arrays.  Keys are case-insensitive (stored lower case).
"""
import re

_NUM = re.compile(r'^[+-]?(\d+\.?\d*|\.\d+)([edED][+-]?\d+)?$')


def _strip_comments(text):
    out, q = [], None
    for line in text.splitlines():
        buf = []
        for ch in line:
            if q:
                buf.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                buf.append(ch)
            elif ch == '!':
                break
            else:
                buf.append(ch)
        q = None
        out.append(''.join(buf))
    return '\n'.join(out)


def _tokens(body):
    """Split a group body into tokens: strings, '=', ',', and bare words."""
    toks, i, n = [], 0, len(body)
    while i < n:
        ch = body[i]
        if ch in ' \t\r\n':
            i += 1
        elif ch in '=,':
            toks.append(ch)
            i += 1
        elif ch in "'\"":
            j = body.index(ch, i + 1)
            toks.append(('str', body[i + 1:j]))
            i = j + 1
        else:
            j = i
            while j < n and body[j] not in ' \t\r\n=,\'"':
                j += 1
            toks.append(body[i:j])
            i = j
    return toks


def _value(tok):
    if isinstance(tok, tuple):
        return tok[1]
    t = tok.strip()
    low = t.lower()
    if low in ('.true.', 't', '.t.', 'true'):
        return True
    if low in ('.false.', 'f', '.f.', 'false'):
        return False
    if _NUM.match(t):
        if re.match(r'^[+-]?\d+$', t):
            return int(t)
        return float(low.replace('d', 'e'))
    return t


def parse(text):
    """Return a list of (group_name, dict) in file order."""
    text = _strip_comments(text)
    groups, i, n = [], 0, len(text)
    while True:
        i = text.find('&', i)
        if i < 0:
            break
        m = re.match(r'&(\w+)', text[i:])
        name = m.group(1).lower()
        j, q = i + m.end(), None
        start = j
        while j < n:
            ch = text[j]
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch == '/':
                break
            j += 1
        body = text[start:j]
        i = j + 1
        toks = _tokens(body)
        d, key, vals = {}, None, []
        k = 0
        while k < len(toks):
            t = toks[k]
            if k + 1 < len(toks) and toks[k + 1] == '=' and not isinstance(t, tuple):
                if key is not None:
                    d[key] = vals[0] if len(vals) == 1 else vals
                key, vals = t.lower(), []
                k += 2
                continue
            if t != ',':
                vals.append(_value(t))
            k += 1
        if key is not None:
            d[key] = vals[0] if len(vals) == 1 else (vals if vals else None)
        groups.append((name, d))
    return groups


def groups_named(groups, name):
    return [d for g, d in groups if g == name.lower()]


def group(groups, name):
    found = groups_named(groups, name)
    return found[0] if found else {}
