/* Declarations of the HEALPix C++ types named by the reference translation
   units that the oracle compiles.  Only the pixel-likelihood path runs; every
   other HEALPix entry point below throws, so a stray call cannot go unnoticed. */
#ifndef CG_SHIM_COMMON_H
#define CG_SHIM_COMMON_H
#include <complex>
#include <vector>
#include <string>
#include <stdexcept>
#include <cstddef>

#include "../../healpix_pix.h"

typedef std::size_t tsize;
enum Healpix_Ordering_Scheme { RING, NEST };
enum nside_dummy { SET_NSIDE };

inline void cg_shim_unavailable(const char* what)
{
    throw std::runtime_error(std::string("HEALPix shim: ") + what + " is not available in the oracle build");
}

template<typename T> class xcomplex : public std::complex<T>
{
public:
    xcomplex() : std::complex<T>() {}
    xcomplex(const T& re, const T& im = T()) : std::complex<T>(re, im) {}
    xcomplex(const std::complex<T>& c) : std::complex<T>(c) {}
    xcomplex conj() const { return xcomplex(std::conj(static_cast<const std::complex<T>&>(*this))); }
};

template<typename T> class arr
{
public:
    arr() {}
    explicit arr(tsize n) : v_(n) {}
    arr(tsize n, const T& val) : v_(n, val) {}
    tsize size() const { return v_.size(); }
    void alloc(tsize n) { v_.assign(n, T()); }
    void fill(const T& val) { for (auto& x : v_) x = val; }
    T& operator[](tsize i) { return v_[i]; }
    const T& operator[](tsize i) const { return v_[i]; }
private:
    std::vector<T> v_;
};

template<typename T> class arr2
{
public:
    arr2() : n1_(0), n2_(0) {}
    arr2(tsize n1, tsize n2) : n1_(n1), n2_(n2), v_(n1 * n2) {}
    T* operator[](tsize i) { return &v_[i * n2_]; }
    const T* operator[](tsize i) const { return &v_[i * n2_]; }
private:
    tsize n1_, n2_;
    std::vector<T> v_;
};

class Healpix_Base
{
public:
    Healpix_Base() : nside_(0), scheme_(RING) {}
    long Nside() const { return nside_; }
    long Npix() const { return 12 * nside_ * nside_; }
    Healpix_Ordering_Scheme Scheme() const { return scheme_; }
    void SetNside(long nside, Healpix_Ordering_Scheme scheme) { nside_ = nside; scheme_ = scheme; }
protected:
    long nside_;
    Healpix_Ordering_Scheme scheme_;
};

template<typename T> class Healpix_Map : public Healpix_Base
{
public:
    Healpix_Map() {}
    Healpix_Map(long nside, Healpix_Ordering_Scheme scheme, nside_dummy) { SetNside(nside, scheme); }
    void SetNside(long nside, Healpix_Ordering_Scheme scheme) { Healpix_Base::SetNside(nside, scheme); map_.assign(Npix(), T()); }
    void fill(const T& val) { for (auto& x : map_) x = val; }
    T& operator[](long i) { return map_[i]; }
    const T& operator[](long i) const { return map_[i]; }
    const std::vector<T>& Map() const { return map_; }
    void Import(const Healpix_Map<T>&) { cg_shim_unavailable("Healpix_Map::Import"); }
    // RING <-> NEST permutation with the shim's pixel functions (Gorski et al. 2005)
    void swap_scheme()
    {
        std::vector<T> out(map_.size());
        for (long i = 0; i < (long)map_.size(); ++i)
            out[scheme_ == RING ? hp_ring2nest(nside_, i) : hp_nest2ring(nside_, i)] = map_[i];
        map_.swap(out);
        scheme_ = scheme_ == RING ? NEST : RING;
    }
    long ang2pix(const struct pointing&) const { cg_shim_unavailable("ang2pix"); return 0; }
    struct pointing pix2ang(long) const;
    T interpolated_value(const struct pointing&) const { cg_shim_unavailable("interpolated_value"); return T(); }
private:
    std::vector<T> map_;
};

template<typename T> class Alm
{
public:
    Alm(int lmax = 0, int mmax = 0) { Set(lmax, mmax); }
    void Set(int lmax, int mmax) { lmax_ = lmax; mmax_ = mmax; a_.assign((tsize)(lmax + 1) * (lmax + 1), T()); }
    int Lmax() const { return lmax_; }
    int Mmax() const { return mmax_; }
    T& operator()(int l, int m) { return a_[(tsize)l * (lmax_ + 1) + m]; }
    const T& operator()(int l, int m) const { return a_[(tsize)l * (lmax_ + 1) + m]; }
    void SetToZero() { for (auto& x : a_) x = T(); }
    bool all_zero() const { for (const auto& x : a_) if (x != T()) return false; return true; }
    template<typename S> void ScaleL(const arr<S>&) { cg_shim_unavailable("Alm::ScaleL"); }
    template<typename S> void Scale(const S& f) { for (auto& x : a_) x *= f; }
private:
    int lmax_, mmax_;
    std::vector<T> a_;
};

struct pointing
{
    double theta, phi;
    pointing() : theta(0), phi(0) {}
    pointing(double t, double p) : theta(t), phi(p) {}
};
template<typename T> pointing Healpix_Map<T>::pix2ang(long) const { cg_shim_unavailable("pix2ang"); return pointing(); }

class rotmatrix
{
public:
    rotmatrix() {}
    rotmatrix(double, double, double, double, double, double, double, double, double) {}
};

class PowSpec
{
public:
    PowSpec() {}
    PowSpec(int, int) {}
    double tt(int) const { cg_shim_unavailable("PowSpec"); return 0; }
    double& tt(int) { cg_shim_unavailable("PowSpec"); static double d; return d; }
};

class fitshandle
{
public:
    fitshandle() {}
};
#endif
