// The drop-in's file formats without a device: CMatrix binary and text files, the
// LegendrePolynomialContainer table file and Utils::readClFromFile, as the reference's callers
// use them (include/c_matrix.hpp:10-83, include/c_matrix_generator.hpp:10-36,
// source/utils.cpp:173-217).
// argv: cmatrix.bin legendre.bin cl_plain.txt dl_with_l.txt outdir
// Writes <out>/c.bin and <out>/c.txt (the binary matrix read and written back, binary and
// text), <out>/c_from_txt.bin (the text file read back, then written binary), <out>/lp.bin (the
// table read and written back); prints the comment, then the two C_l vectors one per line.
#include <cstdio>
#include <string>
#include <vector>

#include <cosmopp_gb300/cosmopp.hpp>

int main(int argc, char** argv)
{
    if (argc < 6) return 2;
    const std::string out = argv[5];
    try {
        CMatrix c(argv[1]);
        c.writeIntoFile((out + "/c.bin").c_str());
        c.writeIntoTextFile((out + "/c.txt").c_str());
        CMatrix t(1);
        t.readFromTextFile((out + "/c.txt").c_str());
        t.writeIntoFile((out + "/c_from_txt.bin").c_str());
        LegendrePolynomialContainer lp(argv[2]);
        lp.writeIntoFile((out + "/lp.bin").c_str());
        std::printf("%s\n", c.comment().c_str());
        std::vector<double> cl;
        Utils::readClFromFile(argv[3], cl);
        for (double v : cl) std::printf("%.17g ", v);
        std::printf("\n");
        Utils::readClFromFile(argv[4], cl, true, true);
        for (double v : cl) std::printf("%.17g ", v);
        std::printf("\n");
        try {
            CMatrix missing("/nonexistent/c.bin");
            std::printf("opened\n");
        } catch (StandardException&) {
            std::printf("raised\n");
        }
    } catch (std::exception& e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 1;
    }
    return 0;
}
