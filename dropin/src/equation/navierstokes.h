//  navierstokes.h -- drop-in NS routines (equation/navierstokes.h of the reference) on the GB300
//  library: the collides run on the device (fused with the recorded Stream and boundary
//  routines), the boundary routines are recorded (see ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace NS {
        //  MacroCollide (navierstokes.h:430-483)
        template<class T, template<class>class P>
        void MacroCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            T *outs[4] = {_rho, _ux, _uy, nullptr};
            pr.collide(PL_NS_COLLIDE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }
        template<class T, template<class>class P>
        void MacroCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, T _viscosity, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            T *outs[4] = {_rho, _ux, _uy, _uz};
            pr.collide(PL_NS_COLLIDE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }

        //  MacroBrinkmanCollide (navierstokes.h:485-546)
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, const T *_alpha, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            T *outs[4] = {_rho, _ux, _uy, nullptr};
            pr.collide(PL_NS_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, T _viscosity, const T *_alpha, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            T *outs[4] = {_rho, _ux, _uy, _uz};
            pr.collide(PL_NS_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }

        //  InitialCondition (navierstokes.h:548-572)
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_rho, const T *_ux, const T *_uy) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> r(_rho, pr.n), x(_ux, pr.n), y(_uy, pr.n);
            std::vector<double> z(pr.n, 0.0);
            gpu::ck(pl_init(pr.h, 0, r.p, nullptr, nullptr, nullptr, x.p, y.p, z.data()), "pl_init");
        }
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> r(_rho, pr.n), x(_ux, pr.n), y(_uy, pr.n), z(_uz, pr.n);
            gpu::ck(pl_init(pr.h, 0, r.p, nullptr, nullptr, nullptr, x.p, y.p, z.p), "pl_init");
        }

        //  BoundaryConditionSetU (navierstokes.h:91-257, 573-591): Zou-He velocity
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetUAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetUAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetUAlongXFace(P<T>& _p, int _i, int _directionx, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetUAlongYFace(P<T>& _p, int _j, int _directiony, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetUAlongZFace(P<T>& _p, int _k, int _directionz, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_U, 2, _k, _directionz, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetU(P<T>& _p, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NS_U, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
            });
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetU(P<T>& _p, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NS_U, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc, _uzbc);
            });
        }

        //  BoundaryConditionSetRho (navierstokes.h:258-426, 593-612): Zou-He pressure
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRhoAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRhoAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetRhoAlongXFace(P<T>& _p, int _i, int _directionx, Fv0 _rhobc, Fv1 _usbc, Fv2 _utbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc, _utbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetRhoAlongYFace(P<T>& _p, int _j, int _directiony, Fv0 _rhobc, Fv1 _usbc, Fv2 _utbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc, _utbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetRhoAlongZFace(P<T>& _p, int _k, int _directionz, Fv0 _rhobc, Fv1 _usbc, Fv2 _utbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NS_RHO, 2, _k, _directionz, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc, _utbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRho(P<T>& _p, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NS_RHO, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
            });
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void BoundaryConditionSetRho(P<T>& _p, Fv0 _rhobc, Fv1 _usbc, Fv2 _utbc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NS_RHO, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc, _utbc);
            });
        }
    }
}
