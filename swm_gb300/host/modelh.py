"""Reads the CPP switches of a model.h (include/model.h of the reference).

Only ``#define NAME [VALUE]`` lines outside C comments count, as the Fortran
preprocessor sees them.
"""
import re


def parse_defines(text):
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    out = {}
    for line in text.splitlines():
        m = re.match(r'\s*#\s*define\s+(\w+)(?:\(.*?\))?\s*(.*)$', line)
        if m:
            out[m.group(1)] = m.group(2).strip()
    return out
