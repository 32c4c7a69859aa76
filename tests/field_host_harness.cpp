// Host build of the device field / curve headers, for the CPU test suite:
// the same limb logic and point formulas the kernels use, compiled with g++
// (the portable carry path of gb_field.cuh) so tests can compare them with
// the oracle without a GPU.
#include <string.h>

#include "gb_curve.cuh"

using namespace gb;

extern "C" {

void h_fp_mul(uint64_t *out, const uint64_t *a, const uint64_t *b)
{
    fp_t x, y;
    memcpy(&x, a, 48);
    memcpy(&y, b, 48);
    fp_t r = x * y;
    memcpy(out, &r, 48);
}

void h_fp_inv(uint64_t *out, const uint64_t *a)
{
    fp_t x;
    memcpy(&x, a, 48);
    fp_t r = x.inverse();
    memcpy(out, &r, 48);
}

// the binary-GCD inverse (mont_t::inverse_binary) of Fp and Fr
void h_fp_inv_binary(uint64_t *out, const uint64_t *a)
{
    fp_t x;
    memcpy(&x, a, 48);
    fp_t r = x.inverse_binary();
    memcpy(out, &r, 48);
}

void h_fr_inv_binary(uint64_t *out, const uint64_t *a)
{
    fr_t x;
    memcpy(&x, a, 32);
    fr_t r = x.inverse_binary();
    memcpy(out, &r, 32);
}

void h_fr_mul(uint64_t *out, const uint64_t *a, const uint64_t *b)
{
    fr_t x, y;
    memcpy(&x, a, 32);
    memcpy(&y, b, 32);
    fr_t r = x * y;
    memcpy(out, &r, 32);
}

void h_fr_addsub(uint64_t *sum, uint64_t *diff, const uint64_t *a, const uint64_t *b)
{
    fr_t x, y;
    memcpy(&x, a, 32);
    memcpy(&y, b, 32);
    fr_t s = x + y, d = x - y;
    memcpy(sum, &s, 32);
    memcpy(diff, &d, 32);
}

// sum_i (+/-) P_i with XYZZ mixed additions, then the XYZZ-XYZZ add of two
// halves and a doubling check; returns the affine sum and its Jacobian form
void h_xyzz_sum(uint64_t *out_affine, uint64_t *out_jac, const uint64_t *pts, const uint8_t *neg, size_t n)
{
    xyzz_t a = xyzz_t::inf(), b = xyzz_t::inf();
    for (size_t i = 0; i < n; i++) {
        affine_t p;
        memcpy(&p, pts + 12 * i, 96);
        if (i % 2) a.add_affine(p, neg[i] != 0);
        else b.add_affine(p, neg[i] != 0);
    }
    a.add(b);
    affine_t r = a.to_affine();
    memcpy(out_affine, &r, 96);
    jacobian_t j = a.to_jacobian();
    memcpy(out_jac, &j, 144);
}

// [k] P by xyzz_mul_small and by repeated doubling/addition
void h_xyzz_mul_small(uint64_t *out_affine, const uint64_t *pt, uint32_t k)
{
    affine_t p;
    memcpy(&p, pt, 96);
    xyzz_t r = xyzz_mul_small(xyzz_t::from_affine(p), k);
    affine_t a = r.to_affine();
    memcpy(out_affine, &a, 96);
}

}  // extern "C"
