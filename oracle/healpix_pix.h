/* HEALPix pixel-centre geometry (Gorski et al. 2005, ApJ 622, 759, sections 4-5).
 *
 * Test infrastructure: used by the oracle restatement and by the HEALPix shim
 * that lets the reference's own translation units compile without the HEALPix
 * library.  The product library carries its own copy of these formulas
 * (cosmopp_gb300/csrc/cg_geometry.cpp); the two are checked against each other.
 */
#ifndef CG_ORACLE_HEALPIX_PIX_H
#define CG_ORACLE_HEALPIX_PIX_H

#ifdef __cplusplus
extern "C" {
#endif

long hp_nside2npix(long nside);
/* pixel centre (z = cos theta, phi) in RING ordering */
void hp_ring_zphi(long nside, long ipring, double* z, double* phi);
/* NEST index -> RING index */
long hp_nest2ring(long nside, long ipnest);
/* RING index -> NEST index (inverse of hp_nest2ring) */
long hp_ring2nest(long nside, long ipring);
/* theta = acos(z), phi, for both orderings */
void hp_pix2ang_ring(long nside, long ipix, double* theta, double* phi);
void hp_pix2ang_nest(long nside, long ipix, double* theta, double* phi);

#ifdef __cplusplus
}
#endif

#endif
