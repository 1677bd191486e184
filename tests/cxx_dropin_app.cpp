// A caller written against the reference's RealTimeCapon classes (the shape of
// apps/RealTimeCaponTest/App.cpp: a Capon object, getCapon on host buffers,
// then the BuildR and Solver stage objects), compiled against
// include/cos_capon.hpp and linked to libcos_capon.so.  Used by
// tests/test_gpu_cxx_dropin.py.
//
// usage: cxx_dropin_app <cube.bin> <out_dir> Nx Nz M L Yavg d nsys
//   cube.bin: complex64 [Nx][Nz][M]; writes z.bin, w.bin, R.bin (getCapon),
//   Rb.bin (BuildR::getR), xs.bin (Solver::solve of the first nsys R
//   matrices with b = 1) and prints the three status codes.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cos_capon.hpp"

typedef Complex<float> Cf;

static bool write_all(const std::string &path, const std::vector<Cf> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t n = std::fwrite(v.data(), sizeof(Cf), v.size(), f);
    std::fclose(f);
    return n == v.size();
}

int main(int argc, char **argv)
{
    if (argc != 10) {
        std::fprintf(stderr, "usage: %s cube.bin out_dir Nx Nz M L Yavg d nsys\n", argv[0]);
        return 2;
    }
    const std::string out = argv[2];
    int Nx = std::atoi(argv[3]), Nz = std::atoi(argv[4]), M = std::atoi(argv[5]), L = std::atoi(argv[6]);
    int Yavg = std::atoi(argv[7]);
    float d = (float)std::atof(argv[8]);
    int nsys = std::atoi(argv[9]);
    const size_t npix = (size_t)Nx * (size_t)(Nz - 2 * Yavg);

    std::vector<Cf> x((size_t)Nx * Nz * M);
    FILE *f = std::fopen(argv[1], "rb");
    if (!f || std::fread(x.data(), sizeof(Cf), x.size(), f) != x.size()) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    std::fclose(f);

    // Capon::getCapon with R requested (the COPY_R_DEVICE_HOST build of the reference)
    std::vector<Cf> z(npix), w(npix * L), R(npix * L * L);
    Cf *zp = z.data(), *wp = w.data(), *Rp = R.data(), *xp = x.data();
    int Nb = 0;
    Capon capon;
    const int e1 = capon.getCapon(zp, wp, Rp, xp, d, L, Yavg, M, Nx, Nz, Nb);

    // BuildR::getR from host memory
    std::vector<Cf> Rb(npix * L * L);
    Cf *Rbp = Rb.data();
    bool R_on_gpu = false, x_on_gpu = false;
    BuildR build;
    const int e2 = build.getR(Rbp, xp, d, L, Yavg, M, Nx, Nz, Nb, R_on_gpu, x_on_gpu);

    // Solver::solve on the first nsys covariance matrices, b = 1
    std::vector<Cf> xs((size_t)nsys * L), b((size_t)nsys * L, Cf(1.f, 0.f));
    Cf *xsp = xs.data(), *Ap = Rb.data(), *bp = b.data();
    bool xg = false, Ag = false, bg = false;
    Solver solver;
    const int e3 = solver.solve(xsp, Ap, bp, L, nsys, xg, Ag, bg);

    std::printf("%d %d %d\n", e1, e2, e3);
    const bool ok = write_all(out + "/z.bin", z) && write_all(out + "/w.bin", w) && write_all(out + "/R.bin", R) &&
                    write_all(out + "/Rb.bin", Rb) && write_all(out + "/xs.bin", xs);
    return ok ? 0 : 3;
}
