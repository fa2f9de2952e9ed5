/* Stand-in for cfitsio, just enough for Utils::readPixelWindowFunction.
   It serves one virtual pixel-window table whose temperature and
   polarisation columns are all 1, i.e. "no pixel window": the reference's
   own code then returns the Gaussian beam B_l unchanged. */
#ifndef CG_SHIM_FITSIO_H
#define CG_SHIM_FITSIO_H
#include <cstring>
#include <cstdio>
#include <cstdlib>

typedef long long LONGLONG;
struct fitsfile { int current_hdu; };
enum { FLEN_CARD = 81, READONLY = 0, CASEINSEN = 0, TSTRING = 16 };
static const long cg_fits_rows = 40001;

inline int fits_open_file(fitsfile** f, const char*, int, int* status) { static fitsfile ff; ff.current_hdu = 1; *f = &ff; *status = 0; return 0; }
inline int fits_get_hdrspace(fitsfile*, int* nkeys, int*, int*) { *nkeys = 0; return 0; }
inline int fits_get_num_hdus(fitsfile*, int* n, int*) { *n = 2; return 0; }
inline int fits_movabs_hdu(fitsfile* f, int hdu, int* type, int*) { f->current_hdu = hdu; *type = 2; return 0; }
inline int fits_get_num_cols(fitsfile*, int* n, int*) { *n = 2; return 0; }
inline int fits_get_num_rows(fitsfile*, long* n, int*) { *n = cg_fits_rows; return 0; }
inline int fits_get_colname(fitsfile*, int, char* templ, char* name, int* colnum, int*) { std::strcpy(name, "PIXWIN"); *colnum = std::atoi(templ); return 0; }
inline int fits_get_coltype(fitsfile*, int, int* type, long* repeat, long* width, int*) { *type = TSTRING; *repeat = 1; *width = 8; return 0; }
inline int fits_get_col_display_width(fitsfile*, int, int* w, int*) { *w = 8; return 0; }
inline int fits_read_col(fitsfile*, int, int, LONGLONG, LONGLONG, LONGLONG n, void*, void* out, int* anynul, int*)
{
    char** col = (char**)out;
    for (LONGLONG i = 0; i < n; ++i) std::strcpy(col[i], "1");
    *anynul = 0;
    return 0;
}
inline int fits_close_file(fitsfile*, int*) { return 0; }
inline void fits_report_error(FILE*, int) {}
#endif
