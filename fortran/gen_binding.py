"""Writes fortran/swm_gpu_binding.f90, the ISO_C_BINDING module of the C ABI,
from include/swm_gpu.h: one bind(C) interface per function the header
declares, the header's enums and #defines as named constants, and the
configuration struct as a bind(C) derived type.

Argument mapping: int / int32_t / int64_t / double / uint16_t scalars pass by
value with their C kinds; every pointer passes as type(c_ptr) by value (the
caller gives c_loc of its array, or c_null_ptr), except the configuration,
which passes as the bind(C) type, and the out-pointer of a handle (T **),
which passes as type(c_ptr), intent(out).  Functions returning void become
subroutines.  Run from anywhere:  python fortran/gen_binding.py
(tests/test_fortran_binding.py checks the committed file is current).
"""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), 'include', 'swm_gpu.h')
OUT = os.path.join(HERE, 'swm_gpu_binding.f90')

SCALARS = {'int': 'integer(c_int)', 'int32_t': 'integer(c_int32_t)', 'int64_t': 'integer(c_int64_t)',
           'double': 'real(c_double)', 'uint16_t': 'integer(c_int16_t)'}


def strip_comments(src):
    src = re.sub(r'/\*.*?\*/', ' ', src, flags=re.S)
    return re.sub(r'//[^\n]*', ' ', src)


def parse(src):
    """(functions, enums, defines, config fields) of the header."""
    body = strip_comments(src)
    enums = []
    for blk in re.findall(r'enum\s*\{(.*?)\}\s*;', body, flags=re.S):
        v = -1
        for item in [x.strip() for x in blk.split(',') if x.strip()]:
            if '=' in item:
                name, val = [x.strip() for x in item.split('=')]
                v = int(val)
            else:
                name, v = item, v + 1
            enums.append((name, v))
    defines = re.findall(r'#define\s+(SWM_\w+)\s+(\d+)', src)
    cfg = re.search(r'typedef struct swm_gpu_config \{(.*?)\} swm_gpu_config;', body, flags=re.S).group(1)
    fields = []
    for decl in [d.strip() for d in cfg.split(';') if d.strip()]:
        typ, names = decl.split(None, 1)
        fields.append((typ, [n.strip() for n in names.split(',')]))
    funcs = []
    for m in re.finditer(r'([A-Za-z_][\w \*]*?)\b(\w+)\s*\(([^()]*)\)\s*;', body):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith('typedef') or name in ('swm_gpu_config',):
            continue
        params = []
        if args and args != 'void':
            for a in args.split(','):
                a = a.strip()
                pm = re.match(r'(.*?)(\w+)$', a)
                params.append((pm.group(1).strip(), pm.group(2)))
        funcs.append((ret, name, params))
    return funcs, enums, defines, fields


def fort_arg(ctype, pname):
    """(declaration, kind names used) of one argument."""
    t = ctype.replace('const', '').strip()
    if t == 'swm_gpu_config *':
        return 'type(swm_gpu_config), intent(in) :: %s' % pname, set()
    if t.count('*') == 2:
        return 'type(c_ptr), intent(out) :: %s' % pname, {'c_ptr'}
    if '*' in t:
        return 'type(c_ptr), value :: %s' % pname, {'c_ptr'}
    f = SCALARS[t]
    return '%s, value :: %s' % (f, pname), {f[f.index('(') + 1:-1]}


def fort_name(name):
    # Fortran names: no leading underscore; 'type' etc. are fine as arguments
    return {'type': 'typ', 'out': 'out_', 'in': 'in_'}.get(name, name)


def wrap(line, width=100):
    """A free-form line split with '&' continuations after commas."""
    out = []
    while len(line) > width:
        cut = line.rfind(', ', 0, width)
        if cut < 0:
            break
        out.append(line[:cut + 1] + ' &')
        line = '        ' + line[cut + 2:]
    out.append(line)
    return out


def generate(src):
    funcs, enums, defines, fields = parse(src)
    L = ['! swm_gpu_binding.f90 -- ISO_C_BINDING interfaces of include/swm_gpu.h.',
         '!',
         '! Written by fortran/gen_binding.py from the header; do not edit by hand.',
         '! Every pointer argument is type(c_ptr), value: pass c_loc(array) of the',
         '! Fortran (Nx, Ny) array (column-major = the C [Ny][Nx] layout the ABI',
         '! uses) or c_null_ptr; handles (contexts, ensembles, solvers) are',
         '! type(c_ptr).  Every integer function returns SWM_GPU_OK or an error',
         '! code; c_string(swm_gpu_last_error()) is the message.',
         '! Not compiled here (this image has no Fortran compiler).',
         'module swm_gpu_binding',
         '  use iso_c_binding',
         '  implicit none',
         '']
    for name, v in enums:
        L.append('  integer(c_int), parameter :: %s = %d' % (name, v))
    for name, v in defines:
        L.append('  integer(c_int), parameter :: %s = %s' % (name, v))
    L += ['', '  type, bind(C) :: swm_gpu_config']
    for typ, names in fields:
        kind = SCALARS[typ]
        for k in range(0, len(names), 6):
            L.append('    %s :: %s' % (kind, ', '.join(names[k:k + 6])))
    L += ['  end type swm_gpu_config', '', '  interface']
    for ret, name, params in funcs:
        decls, kinds = [], set()
        for ctype, pname in params:
            d, k = fort_arg(ctype, fort_name(pname))
            decls.append(d)
            kinds |= k
        args = ', '.join(fort_name(p) for _, p in params)
        r = ret.replace('const', '').strip()
        if r == 'void':
            head, tail = 'subroutine %s(%s) bind(C)' % (name, args), 'end subroutine %s' % name
        elif '*' in r:
            head, tail = 'function %s(%s) bind(C) result(res)' % (name, args), 'end function %s' % name
            decls.insert(0, 'type(c_ptr) :: res')
            kinds.add('c_ptr')
        else:
            f = SCALARS[r]
            head, tail = '%s function %s(%s) bind(C)' % (f, name, args), 'end function %s' % name
            kinds.add(f[f.index('(') + 1:-1])
        if any('swm_gpu_config' in d for d in decls):
            kinds.add('swm_gpu_config')
        L.extend(wrap('    ' + head))
        if kinds:
            L.append('      import :: %s' % ', '.join(sorted(kinds)))
        for d in decls:
            L.append('      ' + d)
        L.append('    ' + tail)
    L += ['  end interface', '',
          'contains', '',
          '  ! the NUL-terminated C string p as a Fortran string',
          '  function c_string(p) result(s)',
          '    type(c_ptr), intent(in) :: p',
          '    character(len=:), allocatable :: s',
          '    character(kind=c_char), pointer :: a(:)',
          '    integer :: n',
          '    s = ""',
          '    if (.not. c_associated(p)) return',
          '    call c_f_pointer(p, a, [4096])',
          '    n = 0',
          '    do while (n < 4096)',
          '      if (a(n + 1) == c_null_char) exit',
          '      n = n + 1',
          '    end do',
          '    allocate(character(len=n) :: s)',
          '    s = transfer(a(1:n), s)',
          '  end function c_string',
          '',
          'end module swm_gpu_binding', '']
    return '\n'.join(L)


def main():
    with open(HEADER) as fh:
        text = generate(fh.read())
    with open(OUT, 'w') as fh:
        fh.write(text)
    print(OUT)


if __name__ == '__main__':
    main()
