#include "shim_common.h"
// a rotation maps zero coefficients to zero; anything else needs HEALPix's Wigner rotation
template<typename T> void rotate_alm(Alm<xcomplex<T> >& a, const rotmatrix&) { if (!a.all_zero()) cg_shim_unavailable("rotate_alm"); }
template<typename T> void rotate_alm(Alm<xcomplex<T> >& a, Alm<xcomplex<T> >& b, Alm<xcomplex<T> >& c, const rotmatrix&)
{
    if (!a.all_zero() || !b.all_zero() || !c.all_zero()) cg_shim_unavailable("rotate_alm");
}
template<typename T> void rotate_alm(Alm<xcomplex<T> >&, double, double, double) { cg_shim_unavailable("rotate_alm"); }
template<typename T> void create_alm(const PowSpec&, Alm<xcomplex<T> >&, void*) { cg_shim_unavailable("create_alm"); }
template<typename T> void extract_powspec(const Alm<xcomplex<T> >&, PowSpec&) { cg_shim_unavailable("extract_powspec"); }
