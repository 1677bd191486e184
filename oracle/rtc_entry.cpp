// C entry point into the reference's RealTimeCapon GPU library, for timing it
// beside this project's kernels (test/benchmark infrastructure only; never
// linked into the product).
//
// rtc_get_capon forwards to Capon::getCapon (RealTimeCapon/Capon.cpp:73-152)
// on one process-wide Capon object, as getCaponCUDA.pyx:7 keeps one.  The
// library writes its per-stage wall times (Capon.cpp:446-459) to
// timer_values.txt in the working directory.
#include "Capon.h"

static Capon *g_capon = nullptr;

extern "C" int rtc_get_capon(void *z, void *w, void *R, void *x, float d, int L, int Yavg, int M, int Nx, int Nz,
                             int Nb)
{
    if (!g_capon) g_capon = new Capon();
    Complex<float> *zp = (Complex<float> *)z, *wp = (Complex<float> *)w, *Rp = (Complex<float> *)R,
                   *xp = (Complex<float> *)x;
    return g_capon->getCapon(zp, wp, Rp, xp, d, L, Yavg, M, Nx, Nz, Nb);
}

extern "C" void rtc_release(void)
{
    delete g_capon;
    g_capon = nullptr;
}

#include "BuildR.h"
#include "Solver.h"

// ISolver::solve (Solver.cpp:23-116): batched general systems, host pointers
extern "C" int rtc_solve(void *x, void *A, void *b, int N, int batch)
{
    Solver s;
    Complex<float> *xp = (Complex<float> *)x, *Ap = (Complex<float> *)A, *bp = (Complex<float> *)b;
    bool xg = false, Ag = false, bg = false;
    return s.solve(xp, Ap, bp, N, batch, xg, Ag, bg);
}

// IBuildR::getR (BuildR.cpp:21-106): covariance per pixel, host pointers
extern "C" int rtc_build_r(void *R, void *x, float d, int L, int Yavg, int M, int Nx, int Nz, int Nb)
{
    BuildR br;
    Complex<float> *Rp = (Complex<float> *)R, *xp = (Complex<float> *)x;
    bool Rg = false, xg = false;
    return br.getR(Rp, xp, d, L, Yavg, M, Nx, Nz, Nb, Rg, xg);
}
