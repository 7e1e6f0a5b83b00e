//  vtkxmlexport.h -- drop-in VTKXMLExport (utility/vtkxmlexport.h of the reference): a .pvts
//  index and one .vts piece in ASCII XML, byte-identical to the reference's single-domain
//  output. Values are taken from the functors at the call; formatting and writing run on one
//  background thread per file (vtkio.h), and the files are complete when the exporter is
//  destroyed. One device domain: the particle describes a single piece (mx = my = mz = 1).
#pragma once
#include <cassert>
#include <memory>
#include <string>

#include "vtkio.h"

namespace PANSLBM2 {
    class VTKXMLExport {
public:
        VTKXMLExport() = delete;
        //  the constructor of vtkxmlexport.h:14-88: index, piece header and the point coordinates
        template<class T, template<class>class P>
        VTKXMLExport(P<T>& _p, std::string _fname) {
            assert(_p.mx * _p.my * _p.mz == 1);
            const int nnx = _p.nx + (_p.PEx != _p.mx - 1 ? 1 : 0), nny = _p.ny + (_p.PEy != _p.my - 1 ? 1 : 0);
            const int nnz = _p.nz + (_p.PEz != _p.mz - 1 ? 1 : 0);
            const int ox = _p.offsetx, oy = _p.offsety, oz = _p.offsetz;
            auto I = [](long long v) { std::string s; vtkio::put_int(s, v); return s; };
            const std::string whole = "0 " + I(_p.lx - 1) + " 0 " + I(_p.ly - 1) + " 0 " + I(_p.lz - 1);
            const std::string extent = I(ox) + " " + I(nnx - 1 + ox) + " " + I(oy) + " " + I(nny - 1 + oy) + " " + I(oz) + " " +
                                       I(nnz - 1 + oz);
            if (_p.PEid == 0) {
                const int pos = std::max((int)_fname.rfind('\\'), (int)_fname.rfind('/'));
                const std::string base = _fname.substr(pos != -1 ? pos + 1 : 0);
                std::string head = "<VTKFile type=\"PStructuredGrid\">\n\t<PStructuredGrid GhostLevel=\"0\" WholeExtent=\"" + whole +
                                   "\">\n\t\t<PPoints>\n\t\t\t<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\"/>\n"
                                   "\t\t</PPoints>\n\t\t<Piece Extent=\"" + extent + "\" Source=\"" + base + "_0.vts\"/>\n";
                this->file0.reset(new vtkio::AsyncFile(_fname + ".pvts"));
                auto st = this->pos0;
                this->file0->post([head, st](std::FILE *fp) {
                    *st = (long long)head.size();
                    vtkio::write_at(fp, 0, head + "\t</PStructuredGrid>\n</VTKFile>");
                });
            }
            std::string head = "<VTKFile type=\"StructuredGrid\">\n\t<StructuredGrid WholeExtent=\"" + whole + "\">\n\t\t<Piece Extent=\"" +
                               extent + "\">\n\t\t\t<Points>\n\t\t\t\t<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
            this->file.reset(new vtkio::AsyncFile(_fname + "_" + std::to_string(_p.PEid) + ".vts"));
            auto st = this->pos;
            this->file->post([head, st, nnx, nny, nnz, ox, oy, oz](std::FILE *fp) {
                std::string s = head + vtkio::format_nodes((size_t)nnx * nny * nnz, [&](std::string &o, size_t n) {
                    const long long i = (long long)(n % nnx), j = (long long)((n / nnx) % nny);
                    const long long k = (long long)(n / ((size_t)nnx * nny));
                    o += "\t\t\t\t\t"; vtkio::put_int(o, i + ox); o += ' '; vtkio::put_int(o, j + oy); o += ' ';
                    vtkio::put_int(o, k + oz); o += '\n';
                });
                s += "\t\t\t\t</DataArray>\n\t\t\t</Points>\n";
                *st = (long long)s.size();
                vtkio::write_at(fp, 0, s + "\t\t</Piece>\n\t</StructuredGrid>\n</VTKFile>");
            });
        }
        VTKXMLExport(const VTKXMLExport&) = delete;
        ~VTKXMLExport() {}

        //  AddPointData (vtkxmlexport.h:107-309): 1, 3 or 9 functors, each value converted to T
        template<class T, template<class>class P, class... Fs>
        void AddPointData(P<T>& _p, std::string _label, Fs ..._values) {
            constexpr int cmp = sizeof...(Fs);
            static_assert(cmp == 1 || cmp == 3 || cmp == 9, "AddPointData takes 1, 3 or 9 functors");
            vtkio::host_sync();
            const int nnx = _p.nx + (_p.PEx != _p.mx - 1 ? 1 : 0), nny = _p.ny + (_p.PEy != _p.my - 1 ? 1 : 0);
            const int nnz = _p.nz + (_p.PEz != _p.mz - 1 ? 1 : 0);
            auto v = std::make_shared<std::vector<double>>((size_t)nnx * nny * nnz * cmp);
            size_t o = 0;
            for (int k = 0; k < nnz; ++k)
                for (int j = 0; j < nny; ++j)
                    for (int i = 0; i < nnx; ++i) {
                        const T vals[cmp] = {T(_values(i, j, k))...};
                        for (int c = 0; c < cmp; ++c) (*v)[o++] = (double)vals[c];
                    }
            const bool first = !this->isaddpointdata;
            this->isaddpointdata = true;
            const std::string array = "<DataArray type=\"Float64\" Name=\"" + _label + "\" NumberOfComponents=\"" +
                                      std::to_string(cmp) + "\" format=\"ascii\"";
            if (this->file0) {
                auto st = this->pos0;
                this->file0->post([st, first, array](std::FILE *fp) {
                    std::string s = first ? "\t\t<PPointData>\n" : "";
                    s += "\t\t\t" + array + "/>\n";
                    const long long at = *st;
                    *st += (long long)s.size();
                    vtkio::write_at(fp, at, s + "\t\t</PPointData>\n\t</PStructuredGrid>\n</VTKFile>");
                });
            }
            auto st = this->pos;
            this->file->post([st, first, array, v](std::FILE *fp) {
                std::string s = first ? "\t\t\t<PointData>\n" : "";
                s += "\t\t\t\t" + array + ">\n";
                s += vtkio::format_nodes(v->size() / cmp, [&](std::string &out, size_t node) {
                    out += "\t\t\t\t\t";
                    for (int c = 0; c < cmp; ++c) { vtkio::put(out, (*v)[node * cmp + c]); out += ' '; }
                    out += '\n';
                });
                s += "\t\t\t\t</DataArray>\n";
                const long long at = *st;
                *st += (long long)s.size();
                vtkio::write_at(fp, at, s + "\t\t\t</PointData>\n\t\t</Piece>\n\t</StructuredGrid>\n</VTKFile>");
            });
        }

private:
        //  the reference's addpos0 / addpos, kept by the writer threads
        std::shared_ptr<long long> pos0 = std::make_shared<long long>(0), pos = std::make_shared<long long>(0);
        std::unique_ptr<vtkio::AsyncFile> file0, file;   // destroyed (joined) before pos0 / pos
        bool isaddpointdata = false;
    };
}
