//  vtkxmlimport.h -- drop-in VTKXMLImport (utility/vtkxmlimport.h of the reference): reads point
//  data from a .pvts index and its .vts pieces. Each file is read into memory once and scanned
//  with the reference's line and token rules (vtkio.h); the same arrays come out.
#pragma once
#include <algorithm>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "vtkio.h"

namespace PANSLBM2 {
    class VTKXMLImport {
public:
        VTKXMLImport() = delete;
        //  the constructor of vtkxmlimport.h:14-43: WholeExtent and the piece file names
        VTKXMLImport(std::string _fname) {
            const int sep = std::max((int)_fname.rfind('\\'), (int)_fname.rfind('/'));
            this->fpath = sep != -1 ? _fname.substr(0, sep + 1) : "";
            const std::string s = vtkio::slurp(_fname);
            size_t cur = 0;
            std::string line;
            while (vtkio::getline(s, cur, line)) {
                std::string::size_type k = line.find("WholeExtent");
                if (k != std::string::npos) {
                    line = quoted(line, k);
                    std::istringstream in(line);
                    int x0, x1, y0, y1, z0, z1;
                    in >> x0 >> x1 >> y0 >> y1 >> z0 >> z1;
                    this->nx = x1 - x0 + 1; this->ny = y1 - y0 + 1; this->nz = z1 - z0 + 1;
                }
                k = line.find("Source");
                if (k != std::string::npos) this->fname_vts.push_back(quoted(line, k));
            }
        }
        VTKXMLImport(const VTKXMLImport&) = delete;
        ~VTKXMLImport() {}

        int GetNx() {   return this->nx;    };
        int GetNy() {   return this->ny;    };
        int GetNz() {   return this->nz;    };

        //  GetPoint* (vtkxmlimport.h:100-143): values of each node in the piece's extent
        template<class T, template<class>class P>
        void GetPointScalar(P<T>& _p, std::string _label, T *_v) {
            this->GetPointBase(_label, [&](int i, int j, int k, vtkio::Tokens &t) { t.number(_v[_p.Index(i, j, k)]); });
        }
        template<class T, template<class>class P>
        void GetPointVector(P<T>& _p, std::string _label, T *_vx, T *_vy) {
            this->GetPointBase(_label, [&](int i, int j, int k, vtkio::Tokens &t) {
                const int idx = _p.Index(i, j, k);
                T tmp;
                t.number(_vx[idx]); t.number(_vy[idx]); t.number(tmp);
            });
        }
        template<class T, template<class>class P>
        void GetPointVector(P<T>& _p, std::string _label, T *_vx, T *_vy, T *_vz) {
            this->GetPointBase(_label, [&](int i, int j, int k, vtkio::Tokens &t) {
                const int idx = _p.Index(i, j, k);
                t.number(_vx[idx]); t.number(_vy[idx]); t.number(_vz[idx]);
            });
        }
        template<class T, template<class>class P>
        void GetPointTensor(P<T>& _p, std::string _label, T *_vxx, T *_vxy, T *_vyx, T *_vyy) {
            this->GetPointBase(_label, [&](int i, int j, int k, vtkio::Tokens &t) {
                const int idx = _p.Index(i, j, k);
                T tmp;
                t.number(_vxx[idx]); t.number(_vxy[idx]); t.number(tmp); t.number(_vyx[idx]); t.number(_vyy[idx]);
                for (int m = 0; m < 4; ++m) t.number(tmp);
            });
        }
        template<class T, template<class>class P>
        void GetPointTensor(P<T>& _p, std::string _label, T *_vxx, T *_vxy, T *_vxz, T *_vyx, T *_vyy, T *_vyz, T *_vzx, T *_vzy, T *_vzz) {
            this->GetPointBase(_label, [&](int i, int j, int k, vtkio::Tokens &t) {
                const int idx = _p.Index(i, j, k);
                T *dst[9] = {_vxx + idx, _vxy + idx, _vxz + idx, _vyx + idx, _vyy + idx, _vyz + idx, _vzx + idx, _vzy + idx, _vzz + idx};
                for (T *d : dst) t.number(*d);
            });
        }

private:
        int nx = 0, ny = 0, nz = 0;
        std::string fpath;
        std::vector<std::string> fname_vts;

        //  the text between the first pair of double quotes after position k
        static std::string quoted(const std::string &line, std::string::size_type k) {
            const std::string::size_type a = line.find("\"", k), b = line.find("\"", a + 1);
            return line.substr(a + 1, b - a - 1);
        }

        //  GetPointBase (vtkxmlimport.h:66-98): in each piece, after the line naming _label, one
        //  call per node of the piece's extent; line scanning resumes where the values end
        template<class F>
        void GetPointBase(std::string _label, F _f) {
            for (const auto &fname : this->fname_vts) {
                const std::string s = vtkio::slurp(this->fpath + fname);
                size_t cur = 0;
                std::string line;
                int x0 = 0, x1 = -1, y0 = 0, y1 = -1, z0 = 0, z1 = -1;
                while (vtkio::getline(s, cur, line)) {
                    std::string::size_type k = line.find("Piece Extent");
                    if (k != std::string::npos) {
                        line = quoted(line, k);
                        std::istringstream in(line);
                        in >> x0 >> x1 >> y0 >> y1 >> z0 >> z1;
                    }
                    if (line.find("Name=\"" + _label + "\"") != std::string::npos) {
                        std::cout << "find out: " << _label << " in " << this->fpath + fname << std::endl;
                        vtkio::Tokens t{&s, cur};
                        for (int kk = z0; kk <= z1; ++kk)
                            for (int j = y0; j <= y1; ++j)
                                for (int i = x0; i <= x1; ++i) _f(i, j, kk, t);
                        cur = t.pos;
                    }
                }
            }
        }
    };
}
