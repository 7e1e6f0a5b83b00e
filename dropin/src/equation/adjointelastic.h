//  adjointelastic.h -- drop-in AEL routines (equation/adjointelastic.h of the reference: the
//  adjoint of the elastic model, D2Q9) on the GB300 library. The collides run on the device,
//  fused with the recorded iStream and boundary routines (see ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace AEL {
        //  MacroCollide (adjointelastic.h:96-125)
        template<class T, template<class>class P>
        void MacroCollide(P<T>& _p, T *_irho, T *_imx, T *_imy, T *_isxx, T *_isxy, T *_isyx, T *_isyy, T _tau, const T *_gamma, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_GAMMA, _gamma);
            T *outs[11] = {_irho, nullptr, nullptr, nullptr, _imx, _imy, nullptr, _isxx, _isxy, _isyx, _isyy};
            pr.collide(PL_AEL_COLLIDE, gpu::phys_tau<T>(_tau), _issave, outs, 11, (T *)nullptr);
        }

        //  InitialCondition (adjointelastic.h:127-138)
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_irho, const T *_imx, const T *_imy, const T *_isxx, const T *_isxy, const T *_isyx, const T *_isyy, const T *_gamma) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            pr.input(PL_GAMMA, _gamma);
            gpu::AsDouble<T> r(_irho, pr.n), x(_imx, pr.n), y(_imy, pr.n), a(_isxx, pr.n), b(_isxy, pr.n), c(_isyx, pr.n), d(_isyy, pr.n);
            const double *in[7] = {r.p, x.p, y.p, a.p, b.p, c.p, d.p};
            gpu::ck(pl_init_elastic(pr.h, 1, in), "pl_init_elastic");
        }

        //  iBoundaryConditionSetStress (adjointelastic.h:48-92, 140-147): the traction over the
        //  node's _rho on an edge
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetStressAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _txbc, Fv1 _tybc, const T *_rho, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_AEL_STRESS, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc,
                           gpu::NodeValues<T>(_rho, _p.nx, _p.ny));
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetStressAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _txbc, Fv1 _tybc, const T *_rho, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_AEL_STRESS, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc,
                           gpu::NodeValues<T>(_rho, _p.nx, _p.ny));
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetStress(P<T>& _p, Fv0 _txbc, Fv1 _tybc, const T *_rho, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_AEL_STRESS, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _txbc, _tybc,
                               gpu::NodeValues<T>(_rho, _p.nx, _p.ny));
            });
        }

        //  SensitivityCompliance (adjointelastic.h:149-155), on the device
        template<class T, template<class>class P>
        void SensitivityCompliance(P<T>& _p, T *_dfds, const T *_sxx, const T *_sxy, const T *_syx, const T *_syy, const T *_irho, const T *_isxx, const T *_isxy, const T *_isyx, const T *_isyy) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> a(_sxx, pr.n), b(_sxy, pr.n), c(_syx, pr.n), d(_syy, pr.n), r(_irho, pr.n), e(_isxx, pr.n),
                f(_isxy, pr.n), g(_isyx, pr.n), h(_isyy, pr.n);
            const double *in[9] = {a.p, b.p, c.p, d.p, r.p, e.p, f.p, g.p, h.p};
            std::vector<double> dv(_dfds, _dfds + pr.n);
            gpu::ck(pl_sensitivity_compliance(pr.h, dv.data(), in), "pl_sensitivity_compliance");
            gpu::to_host(_dfds, dv);
        }
    }
}
