// BLS12-381 G1 (y^2 = x^3 + 4 over Fp) point types for the device.
//
//   affine_t : {x, y}, Montgomery; the point at infinity is all-zero
//              (blst_p1_affine convention; (0,0) is not on the curve).
//   jacobian_t : {X, Y, Z}, x = X/Z^2, y = Y/Z^3; infinity has Z = 0
//              (blst_p1 convention, the reference's RawG1Projective,
//              midnight-sppark-msm/src/lib.rs:30-36).
//   xyzz_t   : {X, Y, ZZ, ZZZ}, x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2;
//              infinity has ZZ = 0.  Bucket accumulators use this form
//              because a mixed (xyzz + affine) addition costs 8M + 2S.
//
// Formulas are the published "xyzz" formulas of the Explicit-Formulas
// Database (madd-2008-s, add-2008-s, dbl-2008-s-1, mdbl-2008-s-1), with the
// equal-point and opposite-point cases routed to doubling / infinity so
// every input combination yields the exact group element.
#pragma once

#include "gb_field.cuh"

namespace gb {

struct affine_t {
    fp_t x, y;
    GB_HD bool is_inf() const { return x.is_zero() && y.is_zero(); }
    GB_HD static affine_t inf()
    {
        affine_t r;
        r.x = fp_t::zero();
        r.y = fp_t::zero();
        return r;
    }
};

struct jacobian_t {
    fp_t x, y, z;
};

struct xyzz_t {
    fp_t x, y, zz, zzz;

    GB_HD static xyzz_t inf()
    {
        xyzz_t r;
        r.x = fp_t::one();
        r.y = fp_t::one();
        r.zz = fp_t::zero();
        r.zzz = fp_t::zero();
        return r;
    }
    GB_HD bool is_inf() const { return zz.is_zero(); }

    GB_HD static xyzz_t from_affine(const affine_t &p)
    {
        if (p.is_inf()) return inf();
        xyzz_t r;
        r.x = p.x;
        r.y = p.y;
        r.zz = fp_t::one();
        r.zzz = fp_t::one();
        return r;
    }

    // affine doubling into xyzz (mdbl-2008-s-1)
    GB_COLD static xyzz_t dbl_affine(const fp_t &x, const fp_t &y)
    {
        xyzz_t r;
        if (y.is_zero()) return inf();
        fp_t U = y.dbl();
        fp_t V = U.sqr();
        fp_t W = U * V;
        fp_t S = x * V;
        fp_t xx = x.sqr();
        fp_t M = xx.dbl() + xx;
        r.x = M.sqr() - S.dbl();
        r.y = M * (S - r.x) - W * y;
        r.zz = V;
        r.zzz = W;
        return r;
    }

    // this += (x, y) for an affine point known not to be infinity
    GB_HD void add_affine(const fp_t &px, const fp_t &py)
    {
        if (is_inf()) {
            x = px;
            y = py;
            zz = fp_t::one();
            zzz = fp_t::one();
            return;
        }
        fp_t U2 = px * zz;
        fp_t S2 = py * zzz;
        fp_t P = U2 - x;
        fp_t R = S2 - y;
        if (P.is_zero()) {
            if (R.is_zero()) *this = dbl_affine(px, py);
            else *this = inf();
            return;
        }
        fp_t PP = P.sqr();
        fp_t PPP = P * PP;
        fp_t Q = x * PP;
        fp_t nx = R.sqr() - PPP - Q.dbl();
        y = R * (Q - nx) - y * PPP;
        x = nx;
        zz = zz * PP;
        zzz = zzz * PPP;
    }

    GB_HD void add_affine(const affine_t &p, bool negate)
    {
        if (p.is_inf()) return;
        add_affine(p.x, negate ? -p.y : p.y);
    }

    // dbl-2008-s-1 (a = 0)
    GB_COLD xyzz_t dbl() const
    {
        if (is_inf()) return *this;
        xyzz_t r;
        fp_t U = y.dbl();
        if (U.is_zero()) return inf();
        fp_t V = U.sqr();
        fp_t W = U * V;
        fp_t S = x * V;
        fp_t xx = x.sqr();
        fp_t M = xx.dbl() + xx;
        r.x = M.sqr() - S.dbl();
        r.y = M * (S - r.x) - W * y;
        r.zz = V * zz;
        r.zzz = W * zzz;
        return r;
    }

    // add-2008-s with the doubling / opposite cases
    GB_COLD void add(const xyzz_t &q)
    {
        if (q.is_inf()) return;
        if (is_inf()) { *this = q; return; }
        fp_t U1 = x * q.zz;
        fp_t U2 = q.x * zz;
        fp_t S1 = y * q.zzz;
        fp_t S2 = q.y * zzz;
        fp_t P = U2 - U1;
        fp_t R = S2 - S1;
        if (P.is_zero()) {
            if (R.is_zero()) *this = dbl();
            else *this = inf();
            return;
        }
        fp_t PP = P.sqr();
        fp_t PPP = P * PP;
        fp_t Q = U1 * PP;
        fp_t nx = R.sqr() - PPP - Q.dbl();
        y = R * (Q - nx) - S1 * PPP;
        x = nx;
        zz = zz * q.zz * PP;
        zzz = zzz * q.zzz * PPP;
    }

#if defined(__CUDACC__)
    // The same doubling and addition with the products issued in independent
    // pairs (fp_mul2): 5 and 7 dependent calls instead of 10 and 14, for
    // kernels bound by the latency of one chain of point operations.
    __device__ xyzz_t dbl_lat() const
    {
        if (is_inf()) return *this;
        xyzz_t r;
        fp_t U = y.dbl();
        if (U.is_zero()) return inf();
        fp_pair p1 = fp_mul2(U, U, x, x);  // V = U^2, xx = x^2
        const fp_t V = p1.a;
        fp_t M = p1.b.dbl() + p1.b;
        fp_pair p2 = fp_mul2(U, V, x, V);  // W = U V, S = x V
        const fp_t W = p2.a, S = p2.b;
        fp_pair p3 = fp_mul2(M, M, V, zz);  // M^2, ZZ3
        r.x = p3.a - S.dbl();
        r.zz = p3.b;
        fp_pair p4 = fp_mul2(M, S - r.x, W, y);
        r.y = p4.a - p4.b;
        r.zzz = W * zzz;
        return r;
    }

    __device__ void add_lat(const xyzz_t &q)
    {
        if (q.is_inf()) return;
        if (is_inf()) {
            *this = q;
            return;
        }
        fp_pair u = fp_mul2(x, q.zz, q.x, zz);    // U1, U2
        fp_pair sv = fp_mul2(y, q.zzz, q.y, zzz);  // S1, S2
        fp_t P = u.b - u.a;
        fp_t R = sv.b - sv.a;
        if (P.is_zero()) {
            if (R.is_zero()) *this = dbl_lat();
            else *this = inf();
            return;
        }
        fp_pair pr = fp_mul2(P, P, zz, q.zz);    // PP, ZZ1 ZZ2
        fp_pair pq = fp_mul2(P, pr.a, u.a, pr.a);  // PPP, Q = U1 PP
        fp_pair rz = fp_mul2(R, R, zzz, q.zzz);  // R^2, ZZZ1 ZZZ2
        const fp_t PPP = pq.a, Q = pq.b;
        fp_t nx = rz.a - PPP - Q.dbl();
        fp_pair yy = fp_mul2(R, Q - nx, sv.a, PPP);
        fp_pair zs = fp_mul2(pr.b, pr.a, rz.b, PPP);
        x = nx;
        y = yy.a - yy.b;
        zz = zs.a;
        zzz = zs.b;
    }
#endif

    GB_HD xyzz_t neg() const
    {
        xyzz_t r = *this;
        r.y = -y;
        return r;
    }

    // (X*ZZ^2, Y*ZZZ^2, ZZZ) is a Jacobian representative of the same point
    // (x = X ZZ^2 / ZZZ^2 = X / ZZ and y = Y ZZZ^2 / ZZZ^3 since ZZZ^2 = ZZ^3).
    GB_COLD jacobian_t to_jacobian() const
    {
        jacobian_t r;
        if (is_inf()) {
            r.x = fp_t::one();
            r.y = fp_t::one();
            r.z = fp_t::zero();
            return r;
        }
        r.x = x * zz.sqr();
        r.y = y * zzz.sqr();
        r.z = zzz;
        return r;
    }

    GB_COLD affine_t to_affine() const
    {
        if (is_inf()) return affine_t::inf();
        // 1/ZZZ = (ZZ)... use a single inversion of ZZZ:
        // 1/ZZ = ZZZ^-1 * (ZZZ/ZZ) and ZZZ/ZZ = Z, ZZ = Z^2 -> 1/ZZ = (1/ZZZ)^2 * ZZ
        fp_t izzz = zzz.inverse();
        fp_t iz = izzz * zz;       // 1/Z
        fp_t izz = iz.sqr();        // 1/Z^2
        affine_t r;
        r.x = x * izz;
        r.y = y * izzz;
        return r;
    }
};

// point operations of the latency-bound kernels (GB_XYZZ_LAT_OFF selects
// the one-product-per-call forms for measurement)
#if defined(GB_XYZZ_LAT_OFF) || !defined(__CUDACC__)
#define GB_ADD_LAT add
#define GB_DBL_LAT dbl
#else
#define GB_ADD_LAT add_lat
#define GB_DBL_LAT dbl_lat
#endif

// scalar multiplication by a small unsigned integer k (double-and-add)
GB_COLD xyzz_t xyzz_mul_small(const xyzz_t &p, uint32_t k)
{
    if (k == 0) return xyzz_t::inf();
    int top = 31;
    while (!((k >> top) & 1u)) top--;
    xyzz_t acc = p;
    for (int i = top - 1; i >= 0; i--) {
#if defined(__CUDA_ARCH__) && !defined(GB_XYZZ_LAT_OFF)
        acc = acc.dbl_lat();
        if ((k >> i) & 1u) acc.add_lat(p);
#else
        acc = acc.dbl();
        if ((k >> i) & 1u) acc.add(p);
#endif
    }
    return acc;
}

}  // namespace gb
