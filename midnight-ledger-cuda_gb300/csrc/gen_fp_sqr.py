"""Writes gb_fp_sqr.cuh: the carry-chain rows of the Fp Montgomery squaring.

Step i of the squaring adds a_i * (a_i at word i, then the words of
2 * sum_{j>i} a_j 2^(32 j)), so its even-word row starts at word
J0 = (i + 1) & ~1 instead of word 0.  One asm statement per start word keeps
each row a single uninterrupted carry chain, like the product's rows.

    python gen_fp_sqr.py > gb_fp_sqr.cuh
"""


def row(j0):
    k = (12 - j0) // 2                  # products in the row
    nacc = 13 - j0                      # acc[j0 .. 12]
    lines = []
    for p in range(k):
        lo, hi = 2 * p, 2 * p + 1       # operand numbers of acc[j0 + 2p], acc[j0 + 2p + 1]
        x = nacc + p                    # operand number of x_p
        y = nacc + k                    # operand number of y
        op = "mad.lo.cc" if p == 0 else "madc.lo.cc"
        lines.append('"%s.u32 %%%d, %%%d, %%%d, %%%d;\\n\\t"' % (op, lo, x, y, lo))
        lines.append('"madc.hi.cc.u32 %%%d, %%%d, %%%d, %%%d;\\n\\t"' % (hi, x, y, hi))
    lines.append('"addc.u32 %%%d, %%%d, 0;"' % (nacc - 1, nacc - 1))
    outs = ", ".join('"+r"(acc[%d])' % (j0 + i) for i in range(nacc))
    ins = ", ".join(['"r"(x[%d])' % p for p in range(k)] + ['"r"(y)'])
    body = "\n        ".join(lines)
    return ("template <>\nGB_D void sqr_row12<%d>(uint32_t *acc, const uint32_t *x, uint32_t y)\n{\n"
            "    asm(%s\n        : %s\n        : %s);\n}\n" % (j0, body, outs, ins))


print("// Generated by gen_fp_sqr.py: do not edit.")
print("// acc[J0 .. 12] += sum_p x[p] * y at words J0 + 2p (lo) and J0 + 2p + 1 (hi),")
print("// carry into acc[12]; words below J0 are untouched.")
print("#pragma once")
print("#if defined(__CUDA_ARCH__)")
print("namespace gb {")
print("template <int J0>\nGB_D void sqr_row12(uint32_t *acc, const uint32_t *x, uint32_t y);\n")
for j0 in range(0, 12, 2):
    print(row(j0))
print("}  // namespace gb")
print("#endif")
