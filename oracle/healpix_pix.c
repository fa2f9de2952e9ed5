/* HEALPix pixel-centre geometry, restated from the published formulas of
 * Gorski et al. 2005 (ApJ 622, 759): eqs. (4)-(9) for ring latitudes and
 * longitudes, section 5 for the nested face/(x,y) indexing.
 *
 * Test infrastructure only (the oracle and the reference shim link it).
 */
#include <math.h>
#include "healpix_pix.h"

/* base-face row/column offsets of the 12 HEALPix base pixels (Gorski et al. fig. 4) */
static const int k_face_row[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
static const int k_face_col[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};

static long isqrt_l(long v)
{
    long r = (long)sqrt((double)v + 0.5);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

long hp_nside2npix(long nside) { return 12 * nside * nside; }

/* RING index -> (ring number i in 1..4nside-1, position j in 1..ring length) */
static void ring_ij(long nside, long p, long* iring, long* iphi, long* nr, int* shifted)
{
    const long npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    if (p < ncap) {
        long i = (1 + isqrt_l(1 + 2 * p)) >> 1;
        *iring = i; *iphi = p - 2 * i * (i - 1) + 1; *nr = i; *shifted = 1;
    } else if (p < npix - ncap) {
        long ip = p - ncap, t = ip / (4 * nside);
        *iring = t + nside; *iphi = ip - t * 4 * nside + 1; *nr = nside;
        /* equatorial rings alternate between phi offsets 0 and pi/(4 nside) */
        *shifted = ((*iring + nside) & 1) ? 0 : 1;
    } else {
        long ip = npix - p;
        long i = (1 + isqrt_l(2 * ip - 1)) >> 1;
        *iring = 4 * nside - i; *iphi = 4 * i + 1 - (ip - 2 * i * (i - 1)); *nr = i; *shifted = 1;
    }
}

void hp_ring_zphi(long nside, long p, double* z, double* phi)
{
    long iring, iphi, nr; int shifted;
    ring_ij(nside, p, &iring, &iphi, &nr, &shifted);
    const double pi = 3.141592653589793;
    const double n2 = (double)nside * (double)nside;
    if (iring < nside) {
        *z = 1.0 - (double)(iring * iring) / (3.0 * n2);
    } else if (iring > 3 * nside) {
        long i = 4 * nside - iring;
        *z = -1.0 + (double)(i * i) / (3.0 * n2);
    } else {
        *z = (double)(2 * nside - iring) * 2.0 / (3.0 * (double)nside);
    }
    *phi = ((double)iphi - (shifted ? 0.5 : 1.0)) * pi / (2.0 * (double)nr);
}

long hp_nest2ring(long nside, long pn)
{
    const long npface = nside * nside, npix = 12 * npface, ncap = 2 * nside * (nside - 1);
    const int face = (int)(pn / npface);
    long ipf = pn % npface, ix = 0, iy = 0;
    for (int b = 0; (ipf >> (2 * b)) != 0; ++b) { /* de-interleave the Morton bits */
        ix |= ((ipf >> (2 * b)) & 1L) << b;
        iy |= ((ipf >> (2 * b + 1)) & 1L) << b;
    }
    const long jr = (long)k_face_row[face] * nside - (ix + iy) - 1; /* ring number 1..4nside-1 */
    long nr, before; int kshift;
    if (jr < nside) { nr = jr; before = 2 * nr * (nr - 1); kshift = 0; }
    else if (jr > 3 * nside) { nr = 4 * nside - jr; before = npix - 2 * (nr + 1) * nr; kshift = 0; }
    else { nr = nside; before = ncap + (jr - nside) * 4 * nside; kshift = (int)((jr - nside) & 1); }
    long jp = ((long)k_face_col[face] * nr + (ix - iy) + 1 + kshift) / 2;
    if (jp > 4 * nr) jp -= 4 * nr;
    if (jp < 1) jp += 4 * nr;
    return before + jp - 1;
}

long hp_ring2nest(long nside, long pr)
{
    /* invert hp_nest2ring within the ring's base faces: a ring pixel lies on one
       base face, found from its (ring, position); solve for (x, y) there */
    long iring, iphi, nr; int shifted;
    ring_ij(nside, pr, &iring, &iphi, &nr, &shifted);
    const long npface = nside * nside;
    for (int face = 0; face < 12; ++face) {
        const long irt = (long)k_face_row[face] * nside - iring - 1; /* = ix + iy */
        if (irt < 0 || irt > 2 * nside - 2) continue;
        const int kshift = (iring >= nside && iring <= 3 * nside) ? (int)((iring - nside) & 1) : 0;
        /* jp = (col*nr + (ix-iy) + 1 + kshift)/2 with wrap; try both wrap images */
        for (int w = -1; w <= 1; ++w) {
            const long jp = iphi + w * 4 * nr;
            for (int parity = 0; parity < 2; ++parity) {
                const long jpt = 2 * jp - parity - (long)k_face_col[face] * nr - 1 - kshift; /* ix - iy */
                if (((irt + jpt) & 1L) != 0) continue;
                const long ix = (irt + jpt) / 2, iy = (irt - jpt) / 2;
                if (ix < 0 || iy < 0 || ix >= nside || iy >= nside) continue;
                long ipf = 0;
                for (int b = 0; (ix >> b) != 0 || (iy >> b) != 0; ++b)
                    ipf |= (((ix >> b) & 1L) << (2 * b)) | (((iy >> b) & 1L) << (2 * b + 1));
                const long cand = face * npface + ipf;
                if (hp_nest2ring(nside, cand) == pr) return cand;
            }
        }
    }
    return -1;
}

void hp_pix2ang_ring(long nside, long ipix, double* theta, double* phi)
{
    double z;
    hp_ring_zphi(nside, ipix, &z, phi);
    *theta = acos(z);
}

void hp_pix2ang_nest(long nside, long ipix, double* theta, double* phi)
{
    hp_pix2ang_ring(nside, hp_nest2ring(nside, ipix), theta, phi);
}
