//  vtkexport.h -- drop-in VTKExport (utility/vtkexport.h of the reference): legacy ASCII VTK
//  structured grid, byte-identical to the reference's output. Values are taken from the
//  functors at the call; formatting and writing run on a background thread (vtkio.h), and the
//  file is complete when the exporter is destroyed.
#pragma once
#include <memory>
#include <string>

#include "vtkio.h"

namespace PANSLBM2 {
    class VTKExport {
public:
        VTKExport() = delete;
        VTKExport(std::string _fname, int _nx, int _ny = 1, int _nz = 1, std::string _title = "notitle")
            : nx(_nx), ny(_ny), nz(_nz), file(new vtkio::AsyncFile(_fname)) {
            const int nx_ = _nx, ny_ = _ny, nz_ = _nz;
            std::string head = "# vtk DataFile Version 3.0\n" + _title + "\nASCII\nDATASET\tSTRUCTURED_GRID\nDIMENSIONS\t";
            vtkio::put_int(head, nx_); head += "\t"; vtkio::put_int(head, ny_); head += "\t"; vtkio::put_int(head, nz_);
            head += "\nPOINTS\t";
            vtkio::put_int(head, (long long)nx_ * ny_ * nz_);
            head += "\tfloat\n";
            this->file->post([head, nx_, ny_, nz_](std::FILE *fp) {
                const std::string s = head + vtkio::format_nodes((size_t)nx_ * ny_ * nz_, [&](std::string &o, size_t n) {
                    const long long i = (long long)(n % nx_), j = (long long)((n / nx_) % ny_);
                    const long long k = (long long)(n / ((size_t)nx_ * ny_));
                    vtkio::put_int(o, i); o += '\t'; vtkio::put_int(o, j); o += '\t'; vtkio::put_int(o, k); o += '\n';
                });
                std::fwrite(s.data(), 1, s.size(), fp);
            });
        }
        VTKExport(const VTKExport&) = delete;
        ~VTKExport() {}

        //  AddPointScaler (vtkexport.h:55-73): one value per line
        template<class F>
        void AddPointScaler(std::string _label, F _value) {
            this->emit(this->point_data() + "SCALARS\t" + _label + "\tfloat\nLOOKUP_TABLE\tdefault\n", this->take(_value), 1);
        }
        //  AddPointVector (vtkexport.h:75-93): three tab-separated values per line
        template<class F0, class F1, class F2>
        void AddPointVector(std::string _label, F0 _value0, F1 _value1, F2 _value2) {
            this->emit(this->point_data() + "VECTORS\t" + _label + "\tfloat\n", this->take(_value0, _value1, _value2), 3);
        }
        //  AddPointTensor (vtkexport.h:95-115): three lines of three, then an empty line
        template<class F00, class F01, class F02, class F10, class F11, class F12, class F20, class F21, class F22>
        void AddPointTensor(std::string _label, F00 _v00, F01 _v01, F02 _v02, F10 _v10, F11 _v11, F12 _v12, F20 _v20, F21 _v21, F22 _v22) {
            this->emit(this->point_data() + "TENSORS\t" + _label + "\tfloat\n",
                       this->take(_v00, _v01, _v02, _v10, _v11, _v12, _v20, _v21, _v22), 9);
        }

private:
        const int nx, ny, nz;
        bool isaddpointdata = false;
        std::unique_ptr<vtkio::AsyncFile> file;

        std::string point_data() {
            if (this->isaddpointdata) return std::string();
            this->isaddpointdata = true;
            std::string s = "POINT_DATA\t";
            vtkio::put_int(s, (long long)this->nx * this->ny * this->nz);
            return s + "\n";
        }
        //  the functors' values at every node in (k, j, i) order, taken on the calling thread
        template<class... Fs>
        std::shared_ptr<std::vector<vtkio::Val>> take(Fs... _f) {
            vtkio::host_sync();
            constexpr int cmp = sizeof...(Fs);
            auto v = std::make_shared<std::vector<vtkio::Val>>((size_t)this->nx * this->ny * this->nz * cmp);
            size_t o = 0;
            for (int k = 0; k < this->nz; k++)
                for (int j = 0; j < this->ny; j++)
                    for (int i = 0; i < this->nx; i++) {
                        const vtkio::Val vals[cmp] = {vtkio::val(_f(i, j, k))...};
                        for (int c = 0; c < cmp; ++c) (*v)[o++] = vals[c];
                    }
            return v;
        }
        //  format and append on the writer thread
        void emit(std::string head, std::shared_ptr<std::vector<vtkio::Val>> v, int cmp) {
            this->file->post([head, v, cmp](std::FILE *fp) {
                const std::string s = head + vtkio::format_nodes(v->size() / cmp, [&](std::string &o, size_t node) {
                    const vtkio::Val *p = v->data() + node * cmp;
                    if (cmp == 1) { vtkio::put(o, p[0]); o += '\n'; return; }
                    for (int r = 0; r < cmp / 3; ++r) {
                        vtkio::put(o, p[3 * r]); o += '\t'; vtkio::put(o, p[3 * r + 1]); o += '\t';
                        vtkio::put(o, p[3 * r + 2]); o += '\n';
                    }
                    if (cmp == 9) o += '\n';
                });
                std::fwrite(s.data(), 1, s.size(), fp);
            });
        }
    };
}
