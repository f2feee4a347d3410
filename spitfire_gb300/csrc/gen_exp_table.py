"""Writes exp_table.h: the constants of the table-driven exponential in chem_device.cuh (Tang's method, ACM TOMS
15(2), 1989), computed at 300 bits with mpmath and rounded to the nearest double.

  python spitfire_gb300/csrc/gen_exp_table.py

* kExpInvL = 64/ln 2;
* kExpL1 + kExpL2 = ln 2/64: kExpL1 is ln 2/64 rounded, kExpL2 the rounded remainder;
* kExpTable[2j], kExpTable[2j+1] = head and tail of 2^(j/64), j = 0..63 (head: 2^(j/64) rounded; tail: the
  rounded remainder), interleaved so that one 16-byte load fetches both.
"""
import os

import mpmath as mp


def header_text():
    """The text of exp_table.h."""
    mp.mp.prec = 300
    ln2 = mp.log(2)
    inv_l = float(64 / ln2)
    l1 = float(ln2 / 64)
    l2 = float(ln2 / 64 - mp.mpf(l1))
    tab = []
    for j in range(64):
        s = mp.power(2, mp.mpf(j) / 64)
        hi = float(s)
        tab += [hi, float(s - mp.mpf(hi))]
    lines = ['// Generated by gen_exp_table.py: constants of the table-driven exponential (Tang, ACM TOMS 15(2), 1989),',
             '// computed at 300 bits and rounded to the nearest double.',
             '#pragma once', '',
             'namespace sfgb {', '',
             f'constexpr double kExpInvL = {inv_l.hex()};  // 64 / ln 2',
             f'constexpr double kExpL1 = {l1.hex()};    // ln 2 / 64, rounded',
             f'constexpr double kExpL2 = {l2.hex()};    // ln 2 / 64 - kExpL1, rounded', '',
             '// 2^(j/64) = kExpTable[2j] + kExpTable[2j + 1], j = 0..63',
             'constexpr double kExpTable[128] = {']
    for j in range(64):
        lines.append(f'    {tab[2 * j].hex()}, {tab[2 * j + 1].hex()},')
    lines += ['};', '', '}  // namespace sfgb', '']
    return '\n'.join(lines)


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'exp_table.h')
    with open(out, 'w') as f:
        f.write(header_text())
    print(out)


if __name__ == '__main__':
    main()
