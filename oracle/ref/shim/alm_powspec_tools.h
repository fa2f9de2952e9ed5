#include "shim_common.h"
template<typename T> void rotate_alm(Alm<xcomplex<T> >&, const rotmatrix&) { cg_shim_unavailable("rotate_alm"); }
template<typename T> void rotate_alm(Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, Alm<xcomplex<T> >&, const rotmatrix&) { cg_shim_unavailable("rotate_alm"); }
template<typename T> void rotate_alm(Alm<xcomplex<T> >&, double, double, double) { cg_shim_unavailable("rotate_alm"); }
template<typename T> void create_alm(const PowSpec&, Alm<xcomplex<T> >&, void*) { cg_shim_unavailable("create_alm"); }
template<typename T> void extract_powspec(const Alm<xcomplex<T> >&, PowSpec&) { cg_shim_unavailable("extract_powspec"); }
