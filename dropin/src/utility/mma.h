//  mma.h -- drop-in MMA<T> (utility/mma.h:58-548 of the reference): Svanberg's method of moving
//  asymptotes with the design-variable update on the device (pl_mma_*, FP64), for up to four
//  constraints. The public parameters are read at every UpdateVariables, as the reference reads
//  its members; ImportSetting / ExportSetting keep the reference's text layout.
#pragma once
#include <cmath>
#include <fstream>
#include <string>
#include <vector>

#include "../gpu/runtime.h"

namespace PANSLBM2 {
    template<class T>
    class MMA {
public:
        MMA() = delete;
        MMA(int _n, int _m, T _a0, std::vector<T> _a, std::vector<T> _c, std::vector<T> _d, const std::vector<T>& _xmin, const std::vector<T>& _xmax) :
            epsvalue(1.0e-6), raa0(1.0e-5), albefa(0.1), move(0.5), asyinit(0.5), asydecr(0.7), asyincr(1.2),
            n(_n), m(_m), a0(_a0), a(_a), c(_c), d(_d), xmin(_xmin), xmax(_xmax), previousvalue(T())
        {
            std::vector<double> av(a.begin(), a.end()), cv(c.begin(), c.end()), dv(d.begin(), d.end());
            std::vector<double> lo(xmin.begin(), xmin.end()), hi(xmax.begin(), xmax.end());
            gpu::ck(pl_mma_create(n, m, double(a0), av.data(), cv.data(), dv.data(), lo.data(), hi.data(), &this->h), "pl_mma_create");
        }
        MMA(const MMA<T>&) = delete;
        ~MMA() { pl_mma_destroy(this->h); }

        void ImportSetting(std::string _fname) {
            std::ifstream fin(_fname);
            int k;
            fin >> k >> this->previousvalue >> this->epsvalue;
            fin >> this->raa0 >> this->albefa >> this->move >> this->asyinit >> this->asydecr >> this->asyincr;
            fin >> this->a0;
            for (int i = 0; i < this->m; ++i) fin >> this->a[i] >> this->c[i] >> this->d[i];
            std::vector<double> xkm2(this->n), xkm1(this->n), L(this->n), U(this->n);
            for (int j = 0; j < this->n; ++j) fin >> this->xmin[j] >> this->xmax[j] >> xkm2[j] >> xkm1[j] >> L[j] >> U[j];
            this->recreate();
            gpu::ck(pl_mma_set_state(this->h, k, double(this->previousvalue), xkm2.data(), xkm1.data(), L.data(), U.data()), "pl_mma_set_state");
        }
        void ExportSetting(std::string _fname) {
            int k;
            double prev;
            std::vector<double> xkm2(this->n), xkm1(this->n), L(this->n), U(this->n);
            gpu::ck(pl_mma_get_state(this->h, &k, &prev, xkm2.data(), xkm1.data(), L.data(), U.data()), "pl_mma_get_state");
            std::ofstream fout(_fname);
            fout << k << std::endl << this->previousvalue << std::endl << this->epsvalue << std::endl;
            fout << this->raa0 << std::endl << this->albefa << std::endl << this->move << std::endl;
            fout << this->asyinit << std::endl << this->asydecr << std::endl << this->asyincr << std::endl;
            fout << this->a0 << std::endl;
            for (int i = 0; i < this->m; ++i) fout << this->a[i] << "\t" << this->c[i] << "\t" << this->d[i] << std::endl;
            for (int j = 0; j < this->n; ++j)
                fout << this->xmin[j] << "\t" << this->xmax[j] << "\t" << xkm2[j] << "\t" << xkm1[j] << "\t" << L[j] << "\t" << U[j] << std::endl;
        }

        bool IsConvergence(T _currentf0) {
            return fabs((_currentf0 - this->previousvalue)/(_currentf0 + this->previousvalue)) < this->epsvalue;
        }
        void UpdateVariables(std::vector<T>& _xk, T _f, const std::vector<T>& _dfdx, const std::vector<T>& _g, const std::vector<std::vector<T> >& _dgdx) {
            const double params[7] = {double(this->move), double(this->asyinit), double(this->asydecr), double(this->asyincr),
                                      double(this->albefa), double(this->raa0), double(this->epsvalue)};
            for (int w = 0; w < 7; ++w) gpu::ck(pl_mma_set_param(this->h, w, params[w]), "pl_mma_set_param");
            std::vector<double> x(_xk.begin(), _xk.end()), df(_dfdx.begin(), _dfdx.end()), g(_g.begin(), _g.end());
            std::vector<double> dg((size_t)this->m * this->n);
            for (int i = 0; i < this->m; ++i)
                for (int j = 0; j < this->n; ++j) dg[(size_t)i * this->n + j] = double(_dgdx[i][j]);
            gpu::sync_outputs();
            gpu::ck(pl_mma_update(this->h, x.data(), double(_f), df.data(), g.data(), dg.data()), "pl_mma_update");
            for (int j = 0; j < this->n; ++j) _xk[j] = T(x[j]);
            this->previousvalue = _f;
        }

        T epsvalue, raa0, albefa, move, asyinit, asydecr, asyincr;

private:
        const int n, m;
        T a0;
        std::vector<T> a, c, d, xmin, xmax;
        T previousvalue;
        pl_mma h = nullptr;

        void recreate() {
            pl_mma_destroy(this->h);
            std::vector<double> av(a.begin(), a.end()), cv(c.begin(), c.end()), dv(d.begin(), d.end());
            std::vector<double> lo(xmin.begin(), xmin.end()), hi(xmax.begin(), xmax.end());
            gpu::ck(pl_mma_create(n, m, double(a0), av.data(), cv.data(), dv.data(), lo.data(), hi.data(), &this->h), "pl_mma_create");
        }
    };
}
