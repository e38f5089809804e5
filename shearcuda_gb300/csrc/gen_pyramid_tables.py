"""Generate pyramid_tables.h from the reference's atrousfilters.m.

The tabulated matrices of shearlet_toolbox_1/atrousfilters.m (cases '9-7',
'maxflat', 'pyr', 'pyrexc') are data that define the pyramid filters; this
script reads them from the MATLAB source text and writes them as C arrays so
that no number is retyped.  The mirroring and scaling steps that follow each
table (atrousfilters.m:100-104, 167-175, 198-206, 228-236) are restated in
host_filters.cpp.

Usage: python gen_pyramid_tables.py /path/to/shearlet_toolbox_1/atrousfilters.m
"""
import os
import re
import sys


def _strip(line):
    out, q = [], False
    for ch in line:
        if ch == "'":
            q = not q
        if ch == '%' and not q:
            break
        out.append(ch)
    return ''.join(out)


def parse_case(text, case):
    lines = text.splitlines()
    start = next(i for i, l in enumerate(lines) if re.match(r"\s*case\s+'%s'" % re.escape(case), l)) + 1
    body = []
    for l in lines[start:]:
        if re.match(r"\s*(case\s+'|end\s*$|otherwise)", l):
            break
        body.append(_strip(l))
    joined = ' '.join(l.replace('...', ' ') for l in body)
    mats = {}
    for m in re.finditer(r"(\w+)\s*=\s*\[([^\]]*)\]", joined):
        name, inner = m.group(1), m.group(2)
        if not re.search(r'\d', inner) or re.search(r'[A-Za-z_]\w*\s*\(', inner):
            continue
        rows = [r for r in inner.split(';') if r.strip()]
        mats[name] = [[float(t) for t in r.replace(',', ' ').split()] for r in rows]
    return mats


def main(path):
    text = open(path).read()
    out = ['// Generated by gen_pyramid_tables.py from shearlet_toolbox_1/atrousfilters.m.',
           '// Tabulated filter matrices (before mirroring / scaling), row-major.',
           '#pragma once', '', 'namespace nsst {', '',
           'struct PyrTable { const char* name; int rows[4]; int cols[4]; const double* m[4]; };', '']
    cases = ('9-7', 'maxflat', 'pyr', 'pyrexc')
    ident = {'9-7': 'c97', 'maxflat': 'maxflat', 'pyr': 'pyr', 'pyrexc': 'pyrexc'}
    for case in cases:
        mats = parse_case(text, case)
        for v in ('h0', 'h1', 'g0', 'g1'):
            m = mats[v]
            vals = ', '.join(repr(x) for row in m for x in row)
            out.append('static const double k_%s_%s[] = {%s};' % (ident[case], v, vals))
        out.append('')
    out.append('static const PyrTable k_pyr_tables[] = {')
    for case in cases:
        mats = parse_case(text, case)
        rows = ', '.join(str(len(mats[v])) for v in ('h0', 'h1', 'g0', 'g1'))
        cols = ', '.join(str(len(mats[v][0])) for v in ('h0', 'h1', 'g0', 'g1'))
        ptrs = ', '.join('k_%s_%s' % (ident[case], v) for v in ('h0', 'h1', 'g0', 'g1'))
        out.append('    {"%s", {%s}, {%s}, {%s}},' % (case, rows, cols, ptrs))
    out.append('};')
    out.append('')
    out.append('}  // namespace nsst')
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'pyramid_tables.h')
    with open(dst, 'w') as f:
        f.write('\n'.join(out) + '\n')
    print('wrote', dst)


if __name__ == '__main__':
    # the reference checkout: an argument, $SHEARCUDA_REFERENCE, else `reference` beside the repository
    ref = os.environ.get('SHEARCUDA_REFERENCE') or os.path.join(
        os.path.dirname(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))), 'reference')
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ref, 'shearlet_toolbox_1', 'atrousfilters.m'))
