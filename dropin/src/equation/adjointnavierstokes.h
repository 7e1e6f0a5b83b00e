//  adjointnavierstokes.h -- drop-in ANS (adjoint NS) routines (equation/adjointnavierstokes.h of
//  the reference) on the GB300 library; iStream and the adjoint boundary routines are recorded
//  and run fused with the next adjoint collide (see ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace ANS {
        //  MacroBrinkmanCollide (adjointnavierstokes.h:396-470); _rho, _ux, _uy[, _uz]: the forward solution
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy, T _viscosity, const T *_alpha, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            pr.input(PL_FWD_RHO, _rho);
            pr.input(PL_FWD_UX, _ux);
            pr.input(PL_FWD_UY, _uy);
            T *outs[11] = {_ip, _iux, _iuy, nullptr, _imx, _imy, nullptr, nullptr, nullptr, nullptr, nullptr};
            pr.collide(PL_ANS_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 11, (T *)nullptr);
        }
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz, T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, T _viscosity, const T *_alpha, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            pr.input(PL_FWD_RHO, _rho);
            pr.input(PL_FWD_UX, _ux);
            pr.input(PL_FWD_UY, _uy);
            pr.input(PL_FWD_UZ, _uz);
            T *outs[11] = {_ip, _iux, _iuy, _iuz, _imx, _imy, _imz, nullptr, nullptr, nullptr, nullptr};
            pr.collide(PL_ANS_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 11, (T *)nullptr);
        }

        //  InitialCondition (adjointnavierstokes.h:472-498)
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_ux, const T *_uy, const T *_ip, const T *_iux, const T *_iuy) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> x(_ux, pr.n), y(_uy, pr.n), ip(_ip, pr.n), ix(_iux, pr.n), iy(_iuy, pr.n);
            std::vector<double> z(pr.n, 0.0);
            gpu::ck(pl_init(pr.h, 2, ip.p, ix.p, iy.p, z.data(), x.p, y.p, z.data()), "pl_init");
        }
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_ux, const T *_uy, const T *_uz, const T *_ip, const T *_iux, const T *_iuy, const T *_iuz) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> x(_ux, pr.n), y(_uy, pr.n), z(_uz, pr.n), ip(_ip, pr.n), ix(_iux, pr.n), iy(_iuy, pr.n), iz(_iuz, pr.n);
            gpu::ck(pl_init(pr.h, 2, ip.p, ix.p, iy.p, iz.p, x.p, y.p, z.p), "pl_init");
        }

        //  iBoundaryConditionSetU (adjointnavierstokes.h:96-256, 500-518)
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetUAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _uxbc, Fv1 _uybc, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANS_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetUAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _uxbc, Fv1 _uybc, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANS_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void iBoundaryConditionSetUAlongXFace(P<T>& _p, int _i, int _directionx, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANS_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void iBoundaryConditionSetUAlongYFace(P<T>& _p, int _j, int _directiony, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANS_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void iBoundaryConditionSetUAlongZFace(P<T>& _p, int _k, int _directionz, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANS_U, 2, _k, _directionz, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc, _uzbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void iBoundaryConditionSetU(P<T>& _p, Fv0 _uxbc, Fv1 _uybc, Ff _bctype, T _eps = T()) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_ANS_U, a, pos, d, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc);
            });
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Fv2, class Ff>
        void iBoundaryConditionSetU(P<T>& _p, Fv0 _uxbc, Fv1 _uybc, Fv2 _uzbc, Ff _bctype, T _eps = T()) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_ANS_U, a, pos, d, _bctype, gpu::IN_NONE, nullptr, double(_eps), 0.0, _uxbc, _uybc, _uzbc);
            });
        }

        //  iBoundaryConditionSetRho (adjointnavierstokes.h:257-392, 520-538)
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongXEdge(P<T>& _p, int _i, int _directionx, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongYEdge(P<T>& _p, int _j, int _directiony, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongXFace(P<T>& _p, int _i, int _directionx, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongYFace(P<T>& _p, int _j, int _directiony, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongZFace(P<T>& _p, int _k, int _directionz, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 2, _k, _directionz, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRho2D(P<T>& _p, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) { gpu::record_bc(_p, 0, PL_BC_ANS_RHO, a, pos, d, _bctype, gpu::IN_NONE); });
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRho3D(P<T>& _p, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) { gpu::record_bc(_p, 0, PL_BC_ANS_RHO, a, pos, d, _bctype, gpu::IN_NONE); });
        }

        //  SensitivityBrinkman (adjointnavierstokes.h:540-554)
        template<class T, template<class>class P>
        void SensitivityBrinkman(P<T>& _p, T *_dfds, const T *_ux, const T *_uy, const T *_imx, const T *_imy, const T *_dads) {
            gpu::Pair &pr = gpu::own(_p, 0);
            gpu::sensitivity(pr, 3, _dfds, _dads, (const T *)nullptr, _ux, _uy, (const T *)nullptr, (const T *)nullptr,
                             _imx, _imy, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr,
                             (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const int *)nullptr);
        }
        template<class T, template<class>class P>
        void SensitivityBrinkman(P<T>& _p, T *_dfds, const T *_ux, const T *_uy, const T *_uz, const T *_imx, const T *_imy, const T *_imz, const T *_dads) {
            gpu::Pair &pr = gpu::own(_p, 0);
            gpu::sensitivity(pr, 3, _dfds, _dads, (const T *)nullptr, _ux, _uy, _uz, (const T *)nullptr,
                             _imx, _imy, _imz, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr,
                             (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const int *)nullptr);
        }
    }
}
