#include "shim_common.h"
template<typename T> void read_Healpix_map_from_fits(const std::string&, Healpix_Map<T>&, int = 1, int = 2) { cg_shim_unavailable("read_Healpix_map_from_fits"); }
template<typename T> void write_Healpix_map_to_fits(fitshandle&, const Healpix_Map<T>&, int) { cg_shim_unavailable("write_Healpix_map_to_fits"); }
