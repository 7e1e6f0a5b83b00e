//  vtk_roundtrip.cpp -- writes one legacy VTK file and one .pvts/.vts pair with the VTK
//  exporters, then reads them back with the importers and dumps what was read. Built against
//  the drop-in headers (dropin/src/utility), or against the reference's own headers with
//  -DUSE_REF -I <reference root>, so a test can compare the two byte for byte.
//
//  usage: vtk_roundtrip <outdir> <nx> <ny> <nz>
//  writes <outdir>/legacy.vtk, <outdir>/xml.pvts, <outdir>/xml_0.vts and <outdir>/read.bin
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#ifdef USE_REF
#include "src/utility/vtkexport.h"
#include "src/utility/vtkxmlexport.h"
#include "src/utility/vtkimport.h"
#include "src/utility/vtkxmlimport.h"
#else
#include "../../dropin/src/utility/vtkexport.h"
#include "../../dropin/src/utility/vtkxmlexport.h"
#include "../../dropin/src/utility/vtkimport.h"
#include "../../dropin/src/utility/vtkxmlimport.h"
#endif

using namespace PANSLBM2;

//  the members of a particle the XML exporter and importer read, for one domain
template<class T>
struct Grid {
    int lx, ly, lz, nx, ny, nz;
    int offsetx = 0, offsety = 0, offsetz = 0, PEid = 0, mx = 1, my = 1, mz = 1, PEx = 0, PEy = 0, PEz = 0;
    Grid(int x, int y, int z) : lx(x), ly(y), lz(z), nx(x), ny(y), nz(z) {}
    int Index(int i, int j, int k) const { return i + nx * (j + ny * k); }
};

int main(int argc, char **argv) {
    if (argc != 5) { std::fprintf(stderr, "usage: %s <outdir> <nx> <ny> <nz>\n", argv[0]); return 2; }
    const std::string dir = argv[1];
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    const int n = nx * ny * nz;
    //  values across magnitudes and signs, with zeros and integers among them
    std::vector<std::vector<double>> a(10, std::vector<double>(n));
    unsigned long long s = 12345;
    for (auto &v : a)
        for (int i = 0; i < n; ++i) {
            s = s * 6364136223846793005ULL + 1442695040888963407ULL;
            const double u = (double)(s >> 11) / 9007199254740992.0;
            const int kind = (int)((s >> 3) % 7);
            v[i] = kind == 0 ? 0.0 : kind == 1 ? std::floor(1000 * u - 500) : (u - 0.4) * std::pow(10.0, (int)(20 * u) - 10);
        }
    auto F = [&](int m) { return [&, m](int i, int j, int k) { return a[m][i + nx * (j + ny * k)]; }; };
    {
        VTKExport e(dir + "/legacy.vtk", nx, ny, nz, "roundtrip");
        e.AddPointScaler("s", F(0));
        e.AddPointScaler("flag", [&](int i, int j, int k) { return (i + j + k) % 3; });
        e.AddPointVector("v", F(1), F(2), F(3));
        e.AddPointTensor("t", F(1), F(2), F(3), F(4), F(5), F(6), F(7), F(8), F(9));
    }
    Grid<double> g(nx, ny, nz);
    {
        VTKXMLExport x(g, dir + "/xml");
        x.AddPointData(g, "s", F(0));
        x.AddPointData(g, "v", F(1), F(2), F(3));
        x.AddPointData(g, "t", F(1), F(2), F(3), F(4), F(5), F(6), F(7), F(8), F(9));
    }
    std::vector<std::vector<double>> r(28, std::vector<double>(n, -7.0));
    {
        VTKImport im(dir + "/legacy.vtk");
        std::printf("legacy %d %d %d\n", im.GetNx(), im.GetNy(), im.GetNz());
        im.GetPointScalar("s", r[0].data());
        im.GetPointVector("v", r[1].data(), r[2].data());
        im.GetPointVector("v", r[3].data(), r[4].data(), r[5].data());
        im.GetPointTensor("t", r[6].data(), r[7].data(), r[8].data(), r[9].data());
        im.GetPointTensor("t", r[10].data(), r[11].data(), r[12].data(), r[13].data(), r[14].data(), r[15].data(),
                          r[16].data(), r[17].data(), r[18].data());
        im.GetPointScalar("missing", r[19].data());
    }
    {
        VTKXMLImport xi(dir + "/xml.pvts");
        std::printf("xml %d %d %d\n", xi.GetNx(), xi.GetNy(), xi.GetNz());
        xi.GetPointScalar(g, "s", r[20].data());
        xi.GetPointVector(g, "v", r[21].data(), r[22].data(), r[23].data());
        xi.GetPointTensor(g, "t", r[24].data(), r[25].data(), r[26].data(), r[27].data());
    }
    FILE *fp = std::fopen((dir + "/read.bin").c_str(), "wb");
    if (!fp) return 2;
    for (auto &v : r) std::fwrite(v.data(), sizeof(double), n, fp);
    std::fclose(fp);
    return 0;
}
