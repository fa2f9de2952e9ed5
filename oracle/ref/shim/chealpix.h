/* Shim for the HEALPix C header: only the pixel functions the reference's
   pixel-likelihood path calls, forwarded to the oracle's own restatement of
   the published HEALPix formulas (oracle/healpix_pix.c). */
#ifndef CG_SHIM_CHEALPIX_H
#define CG_SHIM_CHEALPIX_H
#include "../../healpix_pix.h"
inline long nside2npix(const long nside) { return hp_nside2npix(nside); }
inline void pix2ang_nest(long nside, long ipix, double* theta, double* phi) { hp_pix2ang_nest(nside, ipix, theta, phi); }
inline void pix2ang_ring(long nside, long ipix, double* theta, double* phi) { hp_pix2ang_ring(nside, ipix, theta, phi); }
inline void ring2nest(long nside, long ipring, long* ipnest) { *ipnest = hp_ring2nest(nside, ipring); }
inline void nest2ring(long nside, long ipnest, long* ipring) { *ipring = hp_nest2ring(nside, ipnest); }
#include <stdexcept>
inline float* read_healpix_map(const char*, long*, char*, char*)
{
    throw std::runtime_error("HEALPix shim: read_healpix_map (FITS I/O) is not available in the oracle build");
}
#endif
