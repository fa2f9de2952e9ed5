// HEALPix pixel centres and the Gaussian beam, on the host.
//
// Geometry is a once-per-context O(n) step, computed exactly as the reference
// does it (pix2ang, then (sin t cos p, sin t sin p, cos t), source/
// c_matrix_generator.cpp:178-185) with the host libm, so the unit vectors and
// hence every covariance entry match the reference bit for bit.  Pixel
// centres follow Gorski et al. 2005 (ApJ 622, 759): ring latitudes/longitudes
// of eqs. (4)-(9) and the nested face/(x, y) indexing of section 5.
#include <cmath>

#include "cg_internal.h"

namespace {

const int kFaceRow[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
const int kFaceCol[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};
const double kPi = 3.141592653589793;

long isqrt(long v)
{
    long r = (long)std::sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

// RING index -> ring number (1 .. 4 nside - 1), position in the ring (1-based),
// pixels-per-quarter nr, and whether the ring's longitudes are offset by half a pixel
void ring_position(long nside, long p, long& ring, long& pos, long& nr, bool& half)
{
    const long npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    if (p < ncap) {
        const long i = (1 + isqrt(1 + 2 * p)) >> 1;
        ring = i; pos = p - 2 * i * (i - 1) + 1; nr = i; half = true;
    } else if (p < npix - ncap) {
        const long q = p - ncap, t = q / (4 * nside);
        ring = t + nside; pos = q - t * 4 * nside + 1; nr = nside;
        half = ((ring + nside) & 1) == 0;
    } else {
        const long q = npix - p;
        const long i = (1 + isqrt(2 * q - 1)) >> 1;
        ring = 4 * nside - i; pos = 4 * i + 1 - (q - 2 * i * (i - 1)); nr = i; half = true;
    }
}

void ring_z_phi(long nside, long p, double& z, double& phi)
{
    long ring, pos, nr;
    bool half;
    ring_position(nside, p, ring, pos, nr, half);
    const double n2 = (double)nside * (double)nside;
    if (ring < nside) z = 1.0 - (double)(ring * ring) / (3.0 * n2);
    else if (ring > 3 * nside) {
        const long i = 4 * nside - ring;
        z = -1.0 + (double)(i * i) / (3.0 * n2);
    } else z = (double)(2 * nside - ring) * 2.0 / (3.0 * (double)nside);
    phi = ((double)pos - (half ? 0.5 : 1.0)) * kPi / (2.0 * (double)nr);
}

}  // namespace

extern "C" long cg_nside2npix(long nside) { return 12 * nside * nside; }

extern "C" long cg_nest2ring(long nside, long pn)
{
    if (nside <= 0 || pn < 0 || pn >= 12 * nside * nside) return -1;
    const long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
    const int face = (int)(pn / npface);
    long ipf = pn % npface, ix = 0, iy = 0;
    for (int b = 0; (ipf >> (2 * b)) != 0; ++b) {
        ix |= ((ipf >> (2 * b)) & 1L) << b;
        iy |= ((ipf >> (2 * b + 1)) & 1L) << b;
    }
    const long ring = (long)kFaceRow[face] * nside - (ix + iy) - 1;
    long nr, first;
    int shift;
    if (ring < nside) { nr = ring; first = 2 * nr * (nr - 1); shift = 0; }
    else if (ring > 3 * nside) { nr = 4 * nside - ring; first = npix - 2 * (nr + 1) * nr; shift = 0; }
    else { nr = nside; first = ncap + (ring - nside) * 4 * nside; shift = (int)((ring - nside) & 1); }
    long pos = ((long)kFaceCol[face] * nr + (ix - iy) + 1 + shift) / 2;
    if (pos > 4 * nr) pos -= 4 * nr;
    if (pos < 1) pos += 4 * nr;
    return first + pos - 1;
}

extern "C" long cg_ring2nest(long nside, long pr)
{
    if (nside <= 0 || pr < 0 || pr >= 12 * nside * nside) return -1;
    long ring, pos, nr;
    bool half;
    ring_position(nside, pr, ring, pos, nr, half);
    const long npface = nside * nside;
    for (int face = 0; face < 12; ++face) {
        const long sum = (long)kFaceRow[face] * nside - ring - 1;  // ix + iy on this face
        if (sum < 0 || sum > 2 * nside - 2) continue;
        const int shift = (ring >= nside && ring <= 3 * nside) ? (int)((ring - nside) & 1) : 0;
        for (int wrap = -1; wrap <= 1; ++wrap) {
            for (int par = 0; par < 2; ++par) {
                const long diff = 2 * (pos + wrap * 4 * nr) - par - (long)kFaceCol[face] * nr - 1 - shift;
                if (((sum + diff) & 1L) != 0) continue;
                const long ix = (sum + diff) / 2, iy = (sum - diff) / 2;
                if (ix < 0 || iy < 0 || ix >= nside || iy >= nside) continue;
                long ipf = 0;
                for (int b = 0; (ix >> b) != 0 || (iy >> b) != 0; ++b)
                    ipf |= (((ix >> b) & 1L) << (2 * b)) | (((iy >> b) & 1L) << (2 * b + 1));
                const long cand = face * npface + ipf;
                if (cg_nest2ring(nside, cand) == pr) return cand;
            }
        }
    }
    return -1;
}

extern "C" int cg_pix2vec(long nside, int scheme, const int* pix, int n, double* xyz)
{
    if (nside <= 0 || n < 0 || !xyz || (scheme != CG_SCHEME_RING && scheme != CG_SCHEME_NEST)) return CG_ERR_BAD_ARG;
    const long npix = 12 * nside * nside;
    for (int i = 0; i < n; ++i) {
        const long p = pix ? pix[i] : i;
        if (p < 0 || p >= npix) return CG_ERR_BAD_ARG;
        const long ring = (scheme == CG_SCHEME_NEST) ? cg_nest2ring(nside, p) : p;
        double z, phi;
        ring_z_phi(nside, ring, z, phi);
        const double theta = std::acos(z);
        xyz[3 * i + 0] = std::sin(theta) * std::cos(phi);
        xyz[3 * i + 1] = std::sin(theta) * std::sin(phi);
        xyz[3 * i + 2] = std::cos(theta);
    }
    return CG_OK;
}

// Utils::beamFunction (source/utils.cpp:54-64): fwhm in degrees
extern "C" double cg_beam(int l, double fwhm)
{
    if (fwhm == 0) return 1.0;
    const double sigma = std::sqrt(8 * std::log(2.0)) / (fwhm * kPi / 180);
    return std::exp(-l * (l + 1) / (2 * sigma * sigma));
}
