"""Generate wavelet_tables.h (and the oracle's JSON copy) from the reference's
MakeONFilter.m.

The tabulated coefficient rows of shearcuda/MakeONFilter.m (Haar, Beylkin,
Coiflet, Daubechies, Symmlet, Vaidyanathan, Battle) are data that define the
orthonormal QMF filters; this script reads them from the MATLAB source text and
writes them as C arrays so that no number is retyped.  The two steps that
follow the tables in MakeONFilter.m -- the mirror construction of the Battle
filters from their half (lines 283-286) and the normalisation f / norm(f)
(line 289) -- are restated in host_wavelets.cpp and in the oracle.

Usage: python gen_wavelet_tables.py /path/to/shearcuda/MakeONFilter.m
"""
import json
import os
import re
import sys

_NUM = re.compile(r'[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?')


def _strip(line):
    i = line.find('%')
    return line if i < 0 else line[:i]


def parse(text):
    """-> list of (type, par, half, values); par 0 for the unparameterised
    families, half True for the Battle half-filters (variable g)."""
    out = []
    cur_type, cur_par = None, 0
    lines = [_strip(l) for l in text.splitlines()]
    i = 0
    while i < len(lines):
        l = lines[i]
        m = re.search(r"strcmp\(Type,'(\w+)'\)", l)
        if m:
            cur_type, cur_par = m.group(1), 0
        m = re.search(r'\bPar\s*==\s*(\d+)', l)
        if m:
            cur_par = int(m.group(1))
        m = re.match(r'\s*([fg])\s*=\s*\[', l)
        if m and cur_type is not None:
            var = m.group(1)
            body = l[l.index('[') + 1:]
            while ']' not in body:
                i += 1
                body += ' ' + lines[i]
            body = body[:body.index(']')].replace('...', ' ')
            vals = [float(t) for t in _NUM.findall(body)]
            out.append((cur_type, cur_par, var == 'g', vals))
        i += 1
    return out


def main(src):
    text = open(src).read()
    tabs = parse(text)
    here = os.path.dirname(os.path.abspath(__file__))
    hdr = ['// Generated by gen_wavelet_tables.py from shearcuda/MakeONFilter.m.',
           '// Tabulated QMF coefficients before the Battle mirror step and the',
           '// normalisation f / norm(f).',
           '#pragma once', '', 'namespace nsst {', '',
           'struct OnFilterTable { const char* type; int par; int half; int n; const double* v; };', '']
    names = []
    for (t, p, half, v) in tabs:
        nm = 'k_onf_%s_%d' % (t.lower(), p)
        names.append(nm)
        hdr.append('static const double %s[] = {%s};' % (nm, ', '.join(repr(x) for x in v)))
    hdr.append('')
    hdr.append('static const OnFilterTable kOnFilters[] = {')
    for (t, p, half, v), nm in zip(tabs, names):
        hdr.append('    {"%s", %d, %d, %d, %s},' % (t, p, int(half), len(v), nm))
    hdr.append('};')
    hdr.append('static const int kNumOnFilters = %d;' % len(tabs))
    hdr.append('')
    hdr.append('}  // namespace nsst')
    with open(os.path.join(here, 'wavelet_tables.h'), 'w') as f:
        f.write('\n'.join(hdr) + '\n')
    js = [{'type': t, 'par': p, 'half': half, 'values': v} for (t, p, half, v) in tabs]
    with open(os.path.join(here, '..', '..', 'oracle', 'onfilter_tables.json'), 'w') as f:
        json.dump({'source': 'shearcuda/MakeONFilter.m', 'tables': js}, f, indent=0)
        f.write('\n')
    return tabs


if __name__ == '__main__':
    main(sys.argv[1])
