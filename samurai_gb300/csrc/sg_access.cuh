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
// RevAcc applies the transpose of the operator instead: V is a linear form (a
// short list of (element, weight) terms; constants drop out), get(e) is the
// form "1 * element e", and put(e, form) scatters the adjoint of e onto the
// form's elements.  On a frozen mesh every operator of the path is linear in
// the field (the Dirichlet constant is an affine offset with no derivative),
// so a launch's puts are the rows of its matrix, and the adjoint runs the
// launches with RevAcc in reverse order.
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

    // RevAcc: put(e, form) adds w * lam_in[e] to
    // lam_out[j] for every term (j, w) of the form and, for an operator that
    // updates the field in place, clears lam_in[e] (e was overwritten).  Within
    // one launch of the path's operators every element is written at most once
    // and no written element is read, so the transpose of a launch is the set
    // of its puts in any order; the launches themselves run in reverse order.
    template <int CAP>
    struct RevAcc
    {
        using V = LinForm<CAP>;
        double* lam_in;  // adjoint of the elements the operator writes
        double* lam_out; // adjoint of the elements it reads (accumulated)
        int* overflow;   // set when a form overflowed
        int in_place;    // lam_in == lam_out: clear lam_in[e] after scattering it
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
                atomicOr(overflow, 1);
                return;
            }
            const double ld = lam_in[e];
            if (ld != 0.)
            {
                for (int k = 0; k < v.n; ++k)
                {
                    const double t = v.w[k] * ld;
                    if (t != 0.)
                    {
                        atomicAdd(lam_out + v.idx[k], t);
                    }
                }
            }
            if (in_place)
            {
                lam_in[e] = 0.;
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
