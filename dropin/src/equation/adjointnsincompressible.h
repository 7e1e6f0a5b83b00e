//  adjointnsincompressible.h -- drop-in ANSin routines (equation/adjointnsincompressible.h of the
//  reference: the adjoint of the incompressible NS model, D2Q9) on the GB300 library; iStream and
//  the adjoint boundary routines are recorded and run fused with the next adjoint collide (see
//  ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace ANSin {
        //  MacroBrinkmanCollide (adjointnsincompressible.h:143-178); _ux, _uy: the forward solution
        //  (_rho is taken and not read, as in the reference)
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(
            P<T>& _p, const T *_rho, const T *_ux, const T *_uy,
            T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy,
            T _viscosity, const T *_alpha, bool _issave = false
        ) {
            (void)_rho;
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            pr.input(PL_FWD_UX, _ux);
            pr.input(PL_FWD_UY, _uy);
            T *outs[11] = {_ip, _iux, _iuy, nullptr, _imx, _imy, nullptr, nullptr, nullptr, nullptr, nullptr};
            pr.collide(PL_ANSIN_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 11, (T *)nullptr);
        }

        //  InitialCondition (adjointnsincompressible.h:180-192): the velocity is taken and not read
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_ux, const T *_uy, const T *_ip, const T *_iux, const T *_iuy) {
            (void)_ux; (void)_uy;
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> ip(_ip, pr.n), ix(_iux, pr.n), iy(_iuy, pr.n);
            gpu::ck(pl_init(pr.h, 5, ip.p, ix.p, iy.p, nullptr, nullptr, nullptr, nullptr), "pl_init");
        }

        //  iBoundaryConditionSetU (adjointnsincompressible.h:49-92)
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetUAlongXEdge(P<T>& _p, int _i, int _directionx, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANSIN_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, double(_eps));
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetUAlongYEdge(P<T>& _p, int _j, int _directiony, Ff _bctype, T _eps = T()) {
            gpu::record_bc(_p, 0, PL_BC_ANSIN_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, double(_eps));
        }
        //  the reference's whole-boundary form passes side -1 on all four edges
        //  (adjointnsincompressible.h:194-201); kept, so results match it
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetU(P<T>& _p, Ff _bctype, T _eps = T()) {
            iBoundaryConditionSetUAlongXEdge(_p, 0, -1, _bctype, _eps);
            iBoundaryConditionSetUAlongXEdge(_p, _p.lx - 1, -1, _bctype, _eps);
            iBoundaryConditionSetUAlongYEdge(_p, 0, -1, _bctype, _eps);
            iBoundaryConditionSetUAlongYEdge(_p, _p.ly - 1, -1, _bctype, _eps);
        }

        //  iBoundaryConditionSetRho (adjointnsincompressible.h:93-141, 203-209): the same
        //  arithmetic as ANS::iBoundaryConditionSetRho, so the same library op
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongXEdge(P<T>& _p, int _i, int _directionx, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRhoAlongYEdge(P<T>& _p, int _j, int _directiony, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_ANS_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE);
        }
        template<class T, template<class>class P, class Ff>
        void iBoundaryConditionSetRho2D(P<T>& _p, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) { gpu::record_bc(_p, 0, PL_BC_ANS_RHO, a, pos, d, _bctype, gpu::IN_NONE); });
        }

        //  SensitivityBrinkman (adjointnsincompressible.h:212-217): the ANS routine
        template<class T, template<class>class P>
        void SensitivityBrinkman(P<T>& _p, T *_dfds, const T *_ux, const T *_uy, const T *_imx, const T *_imy, const T *_dads) {
            gpu::Pair &pr = gpu::own(_p, 0);
            gpu::sensitivity(pr, 3, _dfds, _dads, (const T *)nullptr, _ux, _uy, (const T *)nullptr, (const T *)nullptr,
                             _imx, _imy, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr,
                             (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const int *)nullptr);
        }
    }
}
