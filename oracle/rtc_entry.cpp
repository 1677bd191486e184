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
