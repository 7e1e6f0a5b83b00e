//  elastic.h -- drop-in EL routines (equation/elastic.h of the reference: the elastic lattice
//  Boltzmann model, D2Q9) on the GB300 library. The collides run on the device, fused with the
//  recorded Stream and boundary routines (see ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace EL {
        //  MacroCollide (elastic.h:109-136): _rho is the density input; u and the stress are saved
        template<class T, template<class>class P>
        void MacroCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_sxx, T *_sxy, T *_syx, T *_syy, T _tau, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_DENSITY, (const T *)_rho);
            T *outs[8] = {nullptr, _ux, _uy, nullptr, _sxx, _sxy, _syx, _syy};
            pr.collide(PL_EL_COLLIDE, gpu::phys_tau<T>(_tau), _issave, outs, 8, (T *)nullptr);
        }

        //  MacroExtendedCollide (elastic.h:138-166): the stress scaled by gamma
        template<class T, template<class>class P>
        void MacroExtendedCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_sxx, T *_sxy, T *_syx, T *_syy, T _tau, const T *_gamma, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_DENSITY, (const T *)_rho);
            pr.input(PL_GAMMA, _gamma);
            T *outs[8] = {nullptr, _ux, _uy, nullptr, _sxx, _sxy, _syx, _syy};
            pr.collide(PL_EL_EXTENDED, gpu::phys_tau<T>(_tau), _issave, outs, 8, (T *)nullptr);
        }

        //  InitialCondition (elastic.h:168-179)
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_sxx, const T *_sxy, const T *_syx, const T *_syy) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> r(_rho, pr.n), x(_ux, pr.n), y(_uy, pr.n), a(_sxx, pr.n), b(_sxy, pr.n), c(_syx, pr.n), d(_syy, pr.n);
            const double *in[7] = {r.p, x.p, y.p, a.p, b.p, c.p, d.p};
            gpu::ck(pl_init_elastic(pr.h, 0, in), "pl_init_elastic");
        }

        //  BoundaryConditionSetStress (elastic.h:60-104, 181-188): traction (tx, ty) on an edge
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetStressAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _txbc, Fv1 _tybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_EL_STRESS, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetStressAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _txbc, Fv1 _tybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_EL_STRESS, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetStress(P<T>& _p, Fv0 _txbc, Fv1 _tybc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_EL_STRESS, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc);
            });
        }
    }
}
