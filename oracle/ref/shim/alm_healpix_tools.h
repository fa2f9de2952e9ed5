#include "shim_common.h"
template<typename T> void alm2map(const Alm<xcomplex<T> >&, Healpix_Map<T>&) { cg_shim_unavailable("alm2map"); }
template<typename T> void alm2map_pol(const Alm<xcomplex<T> >&, const Alm<xcomplex<T> >&, const Alm<xcomplex<T> >&, Healpix_Map<T>&, Healpix_Map<T>&, Healpix_Map<T>&) { cg_shim_unavailable("alm2map_pol"); }
template<typename T> void map2alm(const Healpix_Map<T>&, Alm<xcomplex<T> >&, const arr<double>&, bool = false) { cg_shim_unavailable("map2alm"); }
template<typename T> void map2alm_iter(const Healpix_Map<T>&, Alm<xcomplex<T> >&, int, const arr<double>&) { cg_shim_unavailable("map2alm_iter"); }
template<typename T> void map2alm_pol_iter(const Healpix_Map<T>&, const Healpix_Map<T>&, const Healpix_Map<T>&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, int, const arr<double>&) { cg_shim_unavailable("map2alm_pol_iter"); }
