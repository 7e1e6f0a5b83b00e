//  nsincompressible.h -- drop-in NSin routines (equation/nsincompressible.h of the reference: the
//  incompressible NS model, D2Q9) on the GB300 library. The collides run on the device, fused
//  with the recorded Stream and boundary routines (see ../gpu/runtime.h).
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace NSin {
        //  MacroCollide (nsincompressible.h:144-169)
        template<class T, template<class>class P>
        void MacroCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            T *outs[4] = {_rho, _ux, _uy, nullptr};
            pr.collide(PL_NSIN_COLLIDE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }

        //  MacroBrinkmanCollide (nsincompressible.h:171-200)
        template<class T, template<class>class P>
        void MacroBrinkmanCollide(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, const T *_alpha, bool _issave = false) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.input(PL_ALPHA, _alpha);
            T *outs[4] = {_rho, _ux, _uy, nullptr};
            pr.collide(PL_NSIN_BRINKMAN, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave, outs, 4, (T *)nullptr);
        }

        //  InitialCondition (nsincompressible.h:202-212)
        template<class T, template<class>class P>
        void InitialCondition(P<T>& _p, const T *_rho, const T *_ux, const T *_uy) {
            gpu::Pair &pr = gpu::own(_p, 0);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> r(_rho, pr.n), x(_ux, pr.n), y(_uy, pr.n);
            gpu::ck(pl_init(pr.h, 4, r.p, nullptr, nullptr, nullptr, x.p, y.p, nullptr), "pl_init");
        }

        //  BoundaryConditionSetU (nsincompressible.h:46-90, 215-222): velocity on an edge
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetUAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NSIN_U, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetUAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NSIN_U, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetU(P<T>& _p, Fv0 _uxbc, Fv1 _uybc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NSIN_U, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _uxbc, _uybc);
            });
        }

        //  BoundaryConditionSetRho (nsincompressible.h:92-140, 224-231): pressure on an edge. The
        //  reference's whole-boundary form misspells its ymin call and does not compile when
        //  instantiated; this one visits the four edges.
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRhoAlongXEdge(P<T>& _p, int _i, int _directionx, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NSIN_RHO, 0, _i, _directionx, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRhoAlongYEdge(P<T>& _p, int _j, int _directiony, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::record_bc(_p, 0, PL_BC_NSIN_RHO, 1, _j, _directiony, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
        }
        template<class T, template<class>class P, class Fv0, class Fv1, class Ff>
        void BoundaryConditionSetRho(P<T>& _p, Fv0 _rhobc, Fv1 _usbc, Ff _bctype) {
            gpu::each_face(_p, [&](int a, int pos, int d) {
                gpu::record_bc(_p, 0, PL_BC_NSIN_RHO, a, pos, d, _bctype, gpu::IN_NONE, nullptr, 0.0, 0.0, _rhobc, _usbc);
            });
        }
    }
}
