#include "shim_common.h"
// Test doubles for a harmonic round trip at one resolution: map2alm_iter keeps the map it was given
// (and leaves the coefficients zero); the next alm2map, onto a map of the same size, with the
// coefficients still zero (any beam ratio applied in between multiplies zeros), writes that map
// back unchanged and records it in cg_shim_synthesised_maps(), so a driver can read the exact maps
// the reference's code went on to use.  Anything else is refused.
inline std::vector<double>& cg_shim_analysed_map() { static std::vector<double> m; return m; }
inline std::vector<std::vector<double> >& cg_shim_synthesised_maps() { static std::vector<std::vector<double> > v; return v; }
template<typename T> void alm2map(const Alm<xcomplex<T> >& a, Healpix_Map<T>& map)
{
    std::vector<double>& kept = cg_shim_analysed_map();
    if (!a.all_zero() || kept.size() != (size_t)map.Npix()) cg_shim_unavailable("alm2map");
    for (long i = 0; i < map.Npix(); ++i) map[i] = (T)kept[i];
    cg_shim_synthesised_maps().push_back(kept);
    kept.clear();
}
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
template<typename T> void map2alm_iter(const Healpix_Map<T>& map, Alm<xcomplex<T> >& a, int, const arr<double>&)
{
    cg_shim_analysed_map().assign(map.Map().begin(), map.Map().end());
    a.SetToZero();
}
template<typename T> void map2alm_pol_iter(const Healpix_Map<T>&, const Healpix_Map<T>&, const Healpix_Map<T>&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, int, const arr<double>&) { cg_shim_unavailable("map2alm_pol_iter"); }
