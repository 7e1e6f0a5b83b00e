//  vtkimport.h -- drop-in VTKImport (utility/vtkimport.h of the reference): reads the point
//  data of a legacy ASCII VTK structured grid. The file is read into memory once and scanned
//  with the reference's token rules (vtkio.h); the same arrays come out.
#pragma once
#include <iostream>
#include <string>

#include "vtkio.h"

namespace PANSLBM2 {
    class VTKImport {
public:
        VTKImport() = delete;
        //  the constructor of vtkimport.h:15-27: DIMENSIONS, POINT_DATA and CELL_DATA counts
        VTKImport(std::string _fname) : text(vtkio::slurp(_fname)) {
            vtkio::Tokens t{&this->text, 0};
            std::string w;
            while (t.word(w)) {
                if (w == "DIMENSIONS") {
                    t.number(this->nx); t.number(this->ny); t.number(this->nz);
                } else if (w == "POINT_DATA") {
                    t.number(this->np);
                } else if (w == "CELL_DATA") {
                    t.number(this->nc);
                }
            }
        }
        VTKImport(const VTKImport&) = delete;
        ~VTKImport() {}

        int GetNx() {   return this->nx;    };
        int GetNy() {   return this->ny;    };
        int GetNz() {   return this->nz;    };

        //  GetPointScalar (vtkimport.h:76-85): after the label, the data type and the lookup table
        template<class T>
        void GetPointScalar(std::string _label, T *_p) {
            this->GetPointBase(_label, "SCALARS", [&](vtkio::Tokens &t) {
                std::string tmp;
                t.word(tmp); t.word(tmp); t.word(tmp);
                for (int i = 0; i < this->np; i++) t.number(_p[i]);
            });
        }
        //  GetPointVector (vtkimport.h:87-107): two or three components of each vector
        template<class T>
        void GetPointVector(std::string _label, T *_px, T *_py) {
            this->GetPointBase(_label, "VECTORS", [&](vtkio::Tokens &t) {
                std::string tmp;
                t.word(tmp);
                for (int i = 0; i < this->np; i++) { t.number(_px[i]); t.number(_py[i]); t.word(tmp); }
            });
        }
        template<class T>
        void GetPointVector(std::string _label, T *_px, T *_py, T *_pz) {
            this->GetPointBase(_label, "VECTORS", [&](vtkio::Tokens &t) {
                std::string tmp;
                t.word(tmp);
                for (int i = 0; i < this->np; i++) { t.number(_px[i]); t.number(_py[i]); t.number(_pz[i]); }
            });
        }
        //  GetPointTensor (vtkimport.h:109-129): the 2D form reads xx xy . yx yy . . . .
        template<class T>
        void GetPointTensor(std::string _label, T *_pxx, T *_pxy, T *_pyx, T *_pyy) {
            this->GetPointBase(_label, "TENSORS", [&](vtkio::Tokens &t) {
                std::string tmp;
                t.word(tmp);
                for (int i = 0; i < this->np; i++) {
                    t.number(_pxx[i]); t.number(_pxy[i]); t.word(tmp); t.number(_pyx[i]); t.number(_pyy[i]);
                    for (int m = 0; m < 4; ++m) t.word(tmp);
                }
            });
        }
        template<class T>
        void GetPointTensor(std::string _label, T *_pxx, T *_pxy, T *_pxz, T *_pyx, T *_pyy, T *_pyz, T *_pzx, T *_pzy, T *_pzz) {
            this->GetPointBase(_label, "TENSORS", [&](vtkio::Tokens &t) {
                std::string tmp;
                t.word(tmp);
                for (int i = 0; i < this->np; i++) {
                    T *dst[9] = {_pxx + i, _pxy + i, _pxz + i, _pyx + i, _pyy + i, _pyz + i, _pzx + i, _pzy + i, _pzz + i};
                    for (T *d : dst) t.number(*d);
                }
            });
        }

private:
        std::string text;
        int nx = 0, ny = 0, nz = 0, np = 0, nc = 0;

        //  GetPointBase (vtkimport.h:53-74): every block `_type _label` inside POINT_DATA, from the top
        template<class F>
        void GetPointBase(std::string _label, std::string _type, F _f) {
            vtkio::Tokens t{&this->text, 0};
            std::string w;
            while (t.word(w)) {
                if (w == "POINT_DATA") {
                    while (t.word(w)) {
                        if (w == _type) {
                            t.word(w);
                            if (w == _label) {
                                std::cout << "Find out \"" << _label << "\"" << std::endl;
                                _f(t);
                            }
                        } else if (w == "CELL_DATA") {
                            break;
                        }
                    }
                } else if (w == "CELL_DATA") {
                    break;
                }
            }
        }
    };
}
