/*
 * cos_capon.hpp -- C++ drop-in for the reference's RealTimeCapon classes,
 * forwarding to the C ABI of cos_capon.h.
 *
 * Provides the interfaces of RealTimeCapon/ICapon.h:9-34, IBuildR.h:43-99 and
 * ISolver.h:9-30 and the concrete classes Capon, BuildR and Solver with the
 * same member signatures, so code written against Capon.h
 * (e.g. apps/RealTimeCaponTest/App.cpp:28-134) compiles unchanged.
 *
 * Complex<float> must be an 8-byte {re, im} float pair, as the reference's
 * framework/lib/Complex.h defines it.  When that header is not included
 * first, a minimal POD with the same layout is declared here.  Define
 * COS_CAPON_HAVE_REFERENCE_INTERFACES when the reference's ICapon.h /
 * IBuildR.h / ISolver.h are already included, to reuse them.
 */
#ifndef COS_CAPON_HPP
#define COS_CAPON_HPP

#include "cos_capon.h"

#ifndef COMPLEX_H
template <class T>
class Complex {
public:
    T re, im;
    Complex() : re(0), im(0) {}
    Complex(T r, T i) : re(r), im(i) {}
};
#endif

#ifndef COS_CAPON_HAVE_REFERENCE_INTERFACES
template <typename C, typename T>
class ICapon {
public:
    virtual ~ICapon() {}
    virtual int getCapon(C *&z, C *&w, C *&R, C *&x, T &d, int &L, int &Yavg, int &M, int &Nx, int &Nz,
                         int &Nb) = 0;
};

template <typename C, typename T>
class IBuildR {
public:
    virtual ~IBuildR() {}
    virtual int getR(C *&R_in, C *&x_in, T &d, int &L, int &Yavg, int &M, int &Nx, int &Nz, int &Nb,
                     bool &R_on_gpu, bool &x_on_gpu) = 0;
};

template <typename C>
class ISolver {
public:
    virtual ~ISolver() {}
    virtual int solve(C *&x, C *&A, C *&b, int &N, int &batch, bool &x_on_gpu, bool &A_on_gpu,
                      bool &b_on_gpu) = 0;
};
#endif

namespace cos_capon_detail {
/* one context per object; created lazily on the calling thread's device */
class Handle {
public:
    Handle() : ctx_(0), err_(0) {}
    ~Handle()
    {
        if (ctx_) cos_capon_destroy(ctx_);
    }
    cos_capon_ctx *get()
    {
        if (!ctx_ && !err_) err_ = cos_capon_create(&ctx_);
        return ctx_;
    }
    int error() const { return err_; }

private:
    Handle(const Handle &);
    Handle &operator=(const Handle &);
    cos_capon_ctx *ctx_;
    int err_;
};
}  // namespace cos_capon_detail

/* Capon::getCapon (Capon.cpp:73-152): host pointers, synchronous, returns a
 * CUDA error number.  R may be NULL. */
class Capon : public ICapon<Complex<float>, float> {
public:
    int getCapon(Complex<float> *&z, Complex<float> *&w, Complex<float> *&R, Complex<float> *&x, float &d, int &L,
                 int &Yavg, int &M, int &Nx, int &Nz, int &Nb)
    {
        cos_capon_ctx *c = h_.get();
        if (!c) return h_.error();
        return cos_capon_get_capon(c, z, w, R, x, d, L, Yavg, M, Nx, Nz, Nb);
    }

private:
    cos_capon_detail::Handle h_;
};

/* BuildR::getR (BuildR.cpp:21-106). */
class BuildR : public IBuildR<Complex<float>, float> {
public:
    int getR(Complex<float> *&R_in, Complex<float> *&x_in, float &d, int &L, int &Yavg, int &M, int &Nx, int &Nz,
             int &Nb, bool &R_on_gpu, bool &x_on_gpu)
    {
        cos_capon_ctx *c = h_.get();
        if (!c) return h_.error();
        return cos_capon_build_r(c, R_in, x_in, d, L, Yavg, M, Nx, Nz, Nb, R_on_gpu ? 1 : 0, x_on_gpu ? 1 : 0);
    }

private:
    cos_capon_detail::Handle h_;
};

/* Solver::solve (Solver.cpp:23-116). */
class Solver : public ISolver<Complex<float> > {
public:
    int solve(Complex<float> *&x, Complex<float> *&A, Complex<float> *&b, int &N, int &batch, bool &x_on_gpu,
              bool &A_on_gpu, bool &b_on_gpu)
    {
        cos_capon_ctx *c = h_.get();
        if (!c) return h_.error();
        return cos_capon_solve(c, x, A, b, N, batch, x_on_gpu ? 1 : 0, A_on_gpu ? 1 : 0, b_on_gpu ? 1 : 0);
    }

private:
    cos_capon_detail::Handle h_;
};

#endif /* COS_CAPON_HPP */
