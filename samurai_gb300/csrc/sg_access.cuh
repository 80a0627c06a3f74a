// Field accessors for the linear FP64 operators of the step (ghost update,
// update_fields).  The kernels of those operators are written once against
// an accessor A:
//   A::V              the value type
//   a.get(e)          the value of element e
//   a.put(e, v)       element e := v
//   A::konst(c)       a constant
// and V supports +, - (binary and unary) and * / by a double.
//
// ValAcc is the plain forward: V = double, reads and writes go to the dense
// slab, and the kernels compile to exactly the arithmetic they spell out.
//
// TapeAcc records the operator instead of applying it: V is a linear form
// (a short list of (element, weight) terms; constants drop out), get(e) is the
// form "1 * element e", and put(e, form) appends one record (e <- j, w) per
// term to a device tape (one record with j = -1 when the form has no term, so
// the transpose still knows that e was overwritten).  On a frozen mesh every
// operator of the path is linear in the field (the Dirichlet constant is an
// affine offset with no derivative), so the tape of a launch is its matrix,
// and the adjoint applies the launches' transposes in reverse order.
#pragma once

#include <cstdint>

namespace sg
{
    struct ValAcc
    {
        using V = double;
        double* u;
        __device__ __forceinline__ double get(long long e) const
        {
            return u[e];
        }
        __device__ __forceinline__ void put(long long e, double v) const
        {
            u[e] = v;
        }
        __device__ __forceinline__ static double konst(double c)
        {
            return c;
        }
    };

    template <int CAP>
    struct LinForm
    {
        int n;        // number of terms; > CAP marks an overflow
        int idx[CAP]; // element indices
        double w[CAP];
    };

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator+(const LinForm<CAP>& a, const LinForm<CAP>& b)
    {
        LinForm<CAP> r;
        r.n = a.n + b.n;
        if (r.n > CAP)
        {
            r.n = CAP + 1;
            return r;
        }
        for (int k = 0; k < a.n; ++k)
        {
            r.idx[k] = a.idx[k];
            r.w[k]   = a.w[k];
        }
        for (int k = 0; k < b.n; ++k)
        {
            r.idx[a.n + k] = b.idx[k];
            r.w[a.n + k]   = b.w[k];
        }
        return r;
    }

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator*(const LinForm<CAP>& a, double s)
    {
        LinForm<CAP> r = a;
        for (int k = 0; k < a.n && k < CAP; ++k)
        {
            r.w[k] = a.w[k] * s;
        }
        return r;
    }

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator*(double s, const LinForm<CAP>& a)
    {
        return a * s;
    }

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator/(const LinForm<CAP>& a, double s)
    {
        return a * (1.0 / s);
    }

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator-(const LinForm<CAP>& a)
    {
        return a * -1.0;
    }

    template <int CAP>
    __device__ __forceinline__ LinForm<CAP> operator-(const LinForm<CAP>& a, const LinForm<CAP>& b)
    {
        return a + (-b);
    }

    // records of a tape, structure of arrays
    struct TapeDev
    {
        int* dst;           // element written
        int* src;           // element read, -1 for "overwritten with a constant"
        double* w;          // weight
        long long* count;   // records appended so far
        long long cap;      // capacity in records
        int* overflow;      // set when a record did not fit or a form overflowed
    };

    template <int CAP>
    struct TapeAcc
    {
        using V = LinForm<CAP>;
        TapeDev t;
        __device__ __forceinline__ V get(long long e) const
        {
            V r;
            r.n      = 1;
            r.idx[0] = static_cast<int>(e);
            r.w[0]   = 1.0;
            return r;
        }
        __device__ __forceinline__ void put(long long e, const V& v) const
        {
            if (v.n > CAP)
            {
                atomicOr(t.overflow, 1);
                return;
            }
            const int n        = v.n > 0 ? v.n : 1;
            const long long at = static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(t.count), static_cast<unsigned long long>(n)));
            if (at + n > t.cap)
            {
                atomicOr(t.overflow, 2);
                return;
            }
            if (v.n == 0)
            {
                t.dst[at] = static_cast<int>(e);
                t.src[at] = -1;
                t.w[at]   = 0.;
                return;
            }
            for (int k = 0; k < v.n; ++k)
            {
                t.dst[at + k] = static_cast<int>(e);
                t.src[at + k] = v.idx[k];
                t.w[at + k]   = v.w[k];
            }
        }
        __device__ __forceinline__ static V konst(double)
        {
            V r;
            r.n = 0;
            return r;
        }
    };

    // form capacity of a dimension: project_bc averages up to 4^dim children
    template <int DIM>
    struct FormCap
    {
        static constexpr int value = (DIM == 2) ? 16 : 64;
    };
} // namespace sg
