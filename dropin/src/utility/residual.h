//  residual.h -- drop-in Residual (utility/residual.h:8-51 of the reference): the relative L2
//  change sqrt(sum |u - up|^2 / sum |u|^2) reduced on the device. When (u, up) are the arrays
//  of the last two saving collides of a lattice, the device reduces its own copies of them;
//  other host arrays are uploaded and reduced on the device of a live lattice.
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace gpu {
        template<class T>
        T residual(const T *const *_a, const T *const *_b, int _ncomp, int _n) {
            auto it = saved_arrays().find(_a[0]);
            if (it != saved_arrays().end() && it->second->n == _n) {
                Pair &pr = *it->second;
                const int fam = pr.residual_family(reinterpret_cast<const void *const *>(_a),
                                                   reinterpret_cast<const void *const *>(_b), _ncomp);
                if (fam >= 0) {
                    pr.flush();
                    double out = 0.0;
                    ck(pl_residual(pr.h, fam, &out), "pl_residual");
                    pr.defer[fam >= 2 ? 1 : 0] = true;   // a residual-driven loop: later saves stay on the device
                    return T(out);
                }
            }
            for (Pair *pr : live_pairs()) {
                if ((long long)_n * 6 > (long long)pr->n * pr->q) continue;   // the library's staging bound
                std::vector<AsDouble<T>> a, b;
                for (int m = 0; m < _ncomp; ++m) { a.emplace_back(_a[m], _n); b.emplace_back(_b[m], _n); }
                const double *pa[3], *pb[3];
                for (int m = 0; m < _ncomp; ++m) { pa[m] = a[m].p; pb[m] = b[m].p; }
                double out = 0.0;
                ck(pl_residual_host(pr->h, _n, _ncomp, pa, pb, &out), "pl_residual_host");
                return T(out);
            }
            die("Residual: no lattice on the device is large enough to stage these arrays");
        }
    }

    template<class T>
    T Residual(const T *_ux, const T *_uxp, int _nxy) {
        const T *a[1] = {_ux}, *b[1] = {_uxp};
        return gpu::residual<T>(a, b, 1, _nxy);
    }

    template<class T>
    T Residual(const T *_ux, const T *_uy, const T *_uxp, const T *_uyp, int _nxy) {
        const T *a[2] = {_ux, _uy}, *b[2] = {_uxp, _uyp};
        return gpu::residual<T>(a, b, 2, _nxy);
    }

    template<class T>
    T Residual(const T *_ux, const T *_uy, const T *_uz, const T *_uxp, const T *_uyp, const T *_uzp, int _nxyz) {
        const T *a[3] = {_ux, _uy, _uz}, *b[3] = {_uxp, _uyp, _uzp};
        return gpu::residual<T>(a, b, 3, _nxyz);
    }
}
