#include "shim_common.h"
#include <fstream>
// Test double: reads a plain-text stand-in for a HEALPix FITS map written by the test driver,
// "nside scheme" (0 = RING, 1 = NEST) then 12 nside^2 values; anything else is refused.
template<typename T> void read_Healpix_map_from_fits(const std::string& path, Healpix_Map<T>& map, int = 1, int = 2)
{
    std::ifstream in(path.c_str());
    long nside = 0;
    int scheme = -1;
    if (!(in >> nside >> scheme) || nside <= 0 || (scheme != 0 && scheme != 1)) cg_shim_unavailable("read_Healpix_map_from_fits");
    map.SetNside(nside, scheme == 1 ? NEST : RING);
    for (long i = 0; i < map.Npix(); ++i)
        if (!(in >> map[i])) cg_shim_unavailable("read_Healpix_map_from_fits (short file)");
}
template<typename T> void write_Healpix_map_to_fits(fitshandle&, const Healpix_Map<T>&, int) { cg_shim_unavailable("write_Healpix_map_to_fits"); }
