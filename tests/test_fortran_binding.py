"""The Fortran binding module fortran/swm_gpu_binding.f90 (host code only,
not compiled here: this image has no Fortran compiler): it is what
fortran/gen_binding.py writes from the current include/swm_gpu.h, it has
one bind(C) interface for every function the header declares, with as many
arguments, and its configuration type has the C struct's fields in order."""
import importlib.util
import os
import re

from test_abi import HEADER, declared_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, 'fortran', 'swm_gpu_binding.f90')


def _gen():
    spec = importlib.util.spec_from_file_location('gen_binding', os.path.join(ROOT, 'fortran', 'gen_binding.py'))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _interfaces(text):
    """name -> argument count of each bind(C) interface in the module."""
    joined = re.sub(r'&\s*\n\s*', '', text)
    out = {}
    for m in re.finditer(r'(?:function|subroutine)\s+(\w+)\(([^)]*)\)\s+bind\(C\)', joined):
        args = [a for a in m.group(2).split(',') if a.strip()]
        out[m.group(1)] = len(args)
    return out


def test_module_is_current():
    with open(HEADER) as fh:
        want = _gen().generate(fh.read())
    with open(F90) as fh:
        assert fh.read() == want, 'run python fortran/gen_binding.py'


def test_every_header_function_has_an_interface():
    with open(F90) as fh:
        got = _interfaces(fh.read())
    with open(HEADER) as fh:
        funcs, _, _, _ = _gen().parse(fh.read())
    assert sorted(got) == declared_functions()
    for _, name, params in funcs:
        assert got[name] == len(params), name


def test_config_type_matches_the_struct():
    from swm_gb300 import _lib
    with open(F90) as fh:
        text = fh.read()
    body = text[text.index('type, bind(C) :: swm_gpu_config'):text.index('end type swm_gpu_config')]
    names = []
    for line in body.splitlines()[1:]:
        if '::' in line:
            names += [n.strip() for n in line.split('::')[1].split(',')]
    assert names == [n for n, _ in _lib.Config._fields_]


def test_lines_fit_free_form():
    with open(F90) as fh:
        assert max(len(l) for l in fh.read().splitlines()) <= 132


def test_shim_calls_declared_entry_points():
    """fortran/swm_gpu_shim.f90 (the GPU bodies of the reference's module
    entry points) calls only functions the header declares, with as many
    arguments as their interfaces take."""
    with open(F90) as fh:
        got = _interfaces(fh.read())
    with open(os.path.join(ROOT, 'fortran', 'swm_gpu_shim.f90')) as fh:
        shim = re.sub(r'!.*', '', fh.read())
    calls = re.findall(r'\b((?:swm_gpu|elsolv_sor_gpu|trc_gpu|swm_helm)_\w+)\(([^()]*(?:\([^()]*\)[^()]*)*)\)', shim)
    assert calls
    for name, args in calls:
        assert name in got, name
        depth, n = 0, 1 if args.strip() else 0
        for ch in args:
            depth += ch == '('
            depth -= ch == ')'
            n += ch == ',' and depth == 0
        assert n == got[name], (name, n, got[name])
