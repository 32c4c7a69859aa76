// Generated by gen_fp_sqr.py: do not edit.
// acc[J0 .. 12] += sum_p x[p] * y at words J0 + 2p (lo) and J0 + 2p + 1 (hi),
// carry into acc[12]; words below J0 are untouched.
#pragma once
#if defined(__CUDA_ARCH__)
namespace gb {
template <int J0>
GB_D void sqr_row12(uint32_t *acc, const uint32_t *x, uint32_t y);

template <>
GB_D void sqr_row12<0>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %13, %19, %0;\n\t"
        "madc.hi.cc.u32 %1, %13, %19, %1;\n\t"
        "madc.lo.cc.u32 %2, %14, %19, %2;\n\t"
        "madc.hi.cc.u32 %3, %14, %19, %3;\n\t"
        "madc.lo.cc.u32 %4, %15, %19, %4;\n\t"
        "madc.hi.cc.u32 %5, %15, %19, %5;\n\t"
        "madc.lo.cc.u32 %6, %16, %19, %6;\n\t"
        "madc.hi.cc.u32 %7, %16, %19, %7;\n\t"
        "madc.lo.cc.u32 %8, %17, %19, %8;\n\t"
        "madc.hi.cc.u32 %9, %17, %19, %9;\n\t"
        "madc.lo.cc.u32 %10, %18, %19, %10;\n\t"
        "madc.hi.cc.u32 %11, %18, %19, %11;\n\t"
        "addc.u32 %12, %12, 0;"
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(y));
}

template <>
GB_D void sqr_row12<2>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %11, %16, %0;\n\t"
        "madc.hi.cc.u32 %1, %11, %16, %1;\n\t"
        "madc.lo.cc.u32 %2, %12, %16, %2;\n\t"
        "madc.hi.cc.u32 %3, %12, %16, %3;\n\t"
        "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
        "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
        "madc.lo.cc.u32 %6, %14, %16, %6;\n\t"
        "madc.hi.cc.u32 %7, %14, %16, %7;\n\t"
        "madc.lo.cc.u32 %8, %15, %16, %8;\n\t"
        "madc.hi.cc.u32 %9, %15, %16, %9;\n\t"
        "addc.u32 %10, %10, 0;"
        : "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(y));
}

template <>
GB_D void sqr_row12<4>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %9, %13, %0;\n\t"
        "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
        "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
        "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
        "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
        "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
        "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
        "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
        "addc.u32 %8, %8, 0;"
        : "+r"(acc[4]), "+r"(acc[5]), "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(y));
}

template <>
GB_D void sqr_row12<6>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %7, %10, %0;\n\t"
        "madc.hi.cc.u32 %1, %7, %10, %1;\n\t"
        "madc.lo.cc.u32 %2, %8, %10, %2;\n\t"
        "madc.hi.cc.u32 %3, %8, %10, %3;\n\t"
        "madc.lo.cc.u32 %4, %9, %10, %4;\n\t"
        "madc.hi.cc.u32 %5, %9, %10, %5;\n\t"
        "addc.u32 %6, %6, 0;"
        : "+r"(acc[6]), "+r"(acc[7]), "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(y));
}

template <>
GB_D void sqr_row12<8>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %5, %7, %0;\n\t"
        "madc.hi.cc.u32 %1, %5, %7, %1;\n\t"
        "madc.lo.cc.u32 %2, %6, %7, %2;\n\t"
        "madc.hi.cc.u32 %3, %6, %7, %3;\n\t"
        "addc.u32 %4, %4, 0;"
        : "+r"(acc[8]), "+r"(acc[9]), "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(x[1]), "r"(y));
}

template <>
GB_D void sqr_row12<10>(uint32_t *acc, const uint32_t *x, uint32_t y)
{
    asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
        "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
        "addc.u32 %2, %2, 0;"
        : "+r"(acc[10]), "+r"(acc[11]), "+r"(acc[12])
        : "r"(x[0]), "r"(y));
}

}  // namespace gb
#endif
