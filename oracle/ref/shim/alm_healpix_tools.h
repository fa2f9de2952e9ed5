#include "shim_common.h"
template<typename T> void alm2map(const Alm<xcomplex<T> >&, Healpix_Map<T>&) { cg_shim_unavailable("alm2map"); }
// zero coefficients synthesise zero maps; anything else needs HEALPix's spherical-harmonic transform
template<typename T> void alm2map_pol(const Alm<xcomplex<T> >& t, const Alm<xcomplex<T> >& e, const Alm<xcomplex<T> >& b,
                                      Healpix_Map<T>& mt, Healpix_Map<T>& mq, Healpix_Map<T>& mu)
{
    if (!t.all_zero() || !e.all_zero() || !b.all_zero()) cg_shim_unavailable("alm2map_pol");
    mt.fill(T());
    mq.fill(T());
    mu.fill(T());
}
template<typename T> void map2alm(const Healpix_Map<T>&, Alm<xcomplex<T> >&, const arr<double>&, bool = false) { cg_shim_unavailable("map2alm"); }
template<typename T> void map2alm_iter(const Healpix_Map<T>&, Alm<xcomplex<T> >&, int, const arr<double>&) { cg_shim_unavailable("map2alm_iter"); }
template<typename T> void map2alm_pol_iter(const Healpix_Map<T>&, const Healpix_Map<T>&, const Healpix_Map<T>&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, int, const arr<double>&) { cg_shim_unavailable("map2alm_pol_iter"); }
