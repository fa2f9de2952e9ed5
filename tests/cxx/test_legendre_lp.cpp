// LegendrePolynomialContainer and the C_l-file overloads of the C++ drop-in, used as the
// reference's callers use them (include/c_matrix_generator.hpp:10-160).
// Input (argv[1]): nside lmax fwhm n, goodPixels[n]; argv[2] = a table file written by the
// reference's own writeIntoFile; argv[3] = a C_l text file (one value per line from l = 0);
// argv[4] = an output folder.
// Writes <out>/lp.bin (the GPU-built table through writeIntoFile), <out>/c_lp.bin (clToCMatrix
// with the reference's table read back by the file constructor) and <out>/c_file.bin
// (clToCMatrix from the C_l file); prints the number of table entries where the file's and
// the GPU's values differ.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include <cosmopp_gb300/cosmopp.hpp>

static void write_packed(const std::string& path, const CMatrix& m)
{
    const int n = m.getNPix();
    std::ofstream out(path, std::ios::binary);
    out.write((const char*)m.data(), sizeof(double) * (size_t)n * (n + 1) / 2);
}

int main(int argc, char** argv)
{
    if (argc < 5) return 2;
    std::ifstream in(argv[1]);
    long nside;
    int lmax, n;
    double fwhm;
    in >> nside >> lmax >> fwhm >> n;
    std::vector<int> good(n);
    for (int& g : good) in >> g;
    const std::string out = argv[4];
    try {
        LegendrePolynomialContainer lp(lmax, nside, &good);
        lp.writeIntoFile((out + "/lp.bin").c_str());
        LegendrePolynomialContainer ref(argv[2]);
        long diff = 0;
        for (int l = 0; l <= lmax; ++l)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i <= j; ++i) diff += lp.value(l, j, i) != ref.value(l, j, i);
        std::vector<double> cl;
        Utils::readClFromFile(argv[3], cl);
        CMatrix* c = CMatrixGenerator::clToCMatrix(cl, nside, fwhm, &good, &ref);
        write_packed(out + "/c_lp.bin", *c);
        delete c;
        c = CMatrixGenerator::clToCMatrix(argv[3], nside, lmax, fwhm, &good);
        write_packed(out + "/c_file.bin", *c);
        delete c;
        std::printf("%ld\n", diff);
        // a table for other pixels is refused, as a mismatched table cannot be meant
        std::vector<int> fewer(good.begin(), good.end() - 1);
        try {
            CMatrixGenerator::clToCMatrix(cl, nside, fwhm, &fewer, &ref);
            std::printf("accepted\n");
        } catch (StandardException&) {
            std::printf("refused\n");
        }
    } catch (std::exception& e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 1;
    }
    return 0;
}
