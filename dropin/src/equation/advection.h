//  advection.h -- drop-in AD (advection-diffusion) routines (equation/advection.h of the
//  reference) on the GB300 library. The coupled collides put the NS particle _p and the AD
//  particle _q on one device handle and run fused with the recorded Stream and boundary routines
//  (see ../gpu/runtime.h).
#pragma once
#include "navierstokes.h"

namespace PANSLBM2 {
    namespace AD {
        namespace detail {
            //  a coupled forward collide: inputs, then the fused step or collide, then the saves
            template<class T, template<class>class P, template<class>class Q>
            void collide(P<T>& _p, Q<T>& _q, int _kind, const pl_phys &_ph, bool _issave, T *_rho, T *_ux, T *_uy, T *_uz,
                         T *_tem, T *_qx, T *_qy, T *_qz, const T *_alpha, const T *_kappa, const T *_beta, T *_g) {
                gpu::Pair &pr = gpu::couple(_p, _q);
                pr.input(PL_ALPHA, _alpha);
                pr.input(PL_KAPPA, _kappa);
                pr.input(PL_BETA, _beta);
                T *outs[8] = {_rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz};
                pr.collide(_kind, _ph, _issave, outs, 8, _g);
            }
        }

        //  MacroCollideForceConvection (advection.h:528-614): no Brinkman term, constant diffusivity
        template<class T, template<class>class P, template<class>class Q>
        void MacroCollideForceConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_FORCE_NOBRINK, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, (T *)nullptr, _tem, _qx, _qy, (T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroCollideForceConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T *_qz, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_FORCE_NOBRINK, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }

        //  MacroCollideNaturalConvection (advection.h:616-712)
        template<class T, template<class>class P, template<class>class Q>
        void MacroCollideNaturalConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T _diffusivity, T _gx, T _gy, T _tem0, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_NATURAL_NOBRINK, gpu::phys<T>(_viscosity, _diffusivity, _gx, _gy, 0, _tem0), _issave,
                            _rho, _ux, _uy, (T *)nullptr, _tem, _qx, _qy, (T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroCollideNaturalConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T *_qz, T _diffusivity, T _gx, T _gy, T _gz, T _tem0, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_NATURAL_NOBRINK, gpu::phys<T>(_viscosity, _diffusivity, _gx, _gy, _gz, _tem0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }

        //  MacroBrinkmanCollideHeatExchange (advection.h:714-810)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideHeatExchange(P<T>& _p, T *_rho, T *_ux, T *_uy, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, const T *_beta, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_HEATEX, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, (T *)nullptr, _tem, _qx, _qy, (T *)nullptr, _alpha, (const T *)nullptr, _beta, (T *)nullptr);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideHeatExchange(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T *_qz, const T *_beta, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AD_HEATEX, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz, _alpha, (const T *)nullptr, _beta, (T *)nullptr);
        }

        //  MacroBrinkmanCollideForceConvection (advection.h:812-926)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideForceConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, const T *_diffusivity, bool _issave = false, T *_g = nullptr) {
            detail::collide(_p, _q, PL_AD_FORCE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, (T *)nullptr, _tem, _qx, _qy, (T *)nullptr, _alpha, _diffusivity, (const T *)nullptr, _g);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideForceConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T *_qz, const T *_diffusivity, bool _issave = false, T *_g = nullptr) {
            detail::collide(_p, _q, PL_AD_FORCE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz, _alpha, _diffusivity, (const T *)nullptr, _g);
        }

        //  MacroBrinkmanCollideNaturalConvection (advection.h:928-1044): the heat-sink drivers' collide
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, const T *_diffusivity, T _gx, T _gy, T _tem0, bool _issave = false, T *_g = nullptr) {
            detail::collide(_p, _q, PL_AD_NATURAL, gpu::phys<T>(_viscosity, 0, _gx, _gy, 0, _tem0), _issave,
                            _rho, _ux, _uy, (T *)nullptr, _tem, _qx, _qy, (T *)nullptr, _alpha, _diffusivity, (const T *)nullptr, _g);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvection(P<T>& _p, T *_rho, T *_ux, T *_uy, T *_uz, const T *_alpha, T _viscosity, Q<T>& _q, T *_tem, T *_qx, T *_qy, T *_qz, const T *_diffusivity, T _gx, T _gy, T _gz, T _tem0, bool _issave = false, T *_g = nullptr) {
            detail::collide(_p, _q, PL_AD_NATURAL, gpu::phys<T>(_viscosity, 0, _gx, _gy, _gz, _tem0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _qx, _qy, _qz, _alpha, _diffusivity, (const T *)nullptr, _g);
        }

        //  InitialCondition (advection.h:1046-1070)
        template<class T, template<class>class Q>
        void InitialCondition(Q<T>& _q, const T *_tem, const T *_ux, const T *_uy) {
            gpu::Pair &pr = gpu::own(_q, 1);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> t(_tem, pr.n), x(_ux, pr.n), y(_uy, pr.n);
            std::vector<double> z(pr.n, 0.0);
            gpu::ck(pl_init(pr.h, 1, t.p, nullptr, nullptr, nullptr, x.p, y.p, z.data()), "pl_init");
        }
        template<class T, template<class>class Q>
        void InitialCondition(Q<T>& _q, const T *_tem, const T *_ux, const T *_uy, const T *_uz) {
            gpu::Pair &pr = gpu::own(_q, 1);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> t(_tem, pr.n), x(_ux, pr.n), y(_uy, pr.n), z(_uz, pr.n);
            gpu::ck(pl_init(pr.h, 1, t.p, nullptr, nullptr, nullptr, x.p, y.p, z.p), "pl_init");
        }

        //  BoundaryConditionSetT (advection.h:97-240, 1072-1091): Dirichlet temperature. The
        //  velocity the routine reads is the one the last saving collide wrote into _ux.
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetTAlongXEdge(Q<T>& _q, int _i, int _directionx, Fv _tembc, const T *_ux, const T *_uy, Ff _bctype) {
            gpu::record_bc(_q, 1, PL_BC_AD_T, 0, _i, _directionx, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetTAlongYEdge(Q<T>& _q, int _j, int _directiony, Fv _tembc, const T *_ux, const T *_uy, Ff _bctype) {
            gpu::record_bc(_q, 1, PL_BC_AD_T, 1, _j, _directiony, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetTAlongXFace(Q<T>& _q, int _i, int _directionx, Fv _tembc, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) {
            gpu::record_bc(_q, 1, PL_BC_AD_T, 0, _i, _directionx, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetTAlongYFace(Q<T>& _q, int _j, int _directiony, Fv _tembc, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) {
            gpu::record_bc(_q, 1, PL_BC_AD_T, 1, _j, _directiony, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetTAlongZFace(Q<T>& _q, int _k, int _directionz, Fv _tembc, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) {
            gpu::record_bc(_q, 1, PL_BC_AD_T, 2, _k, _directionz, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetT(Q<T>& _q, Fv _tembc, const T *_ux, const T *_uy, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) {
                gpu::record_bc(_q, 1, PL_BC_AD_T, a, pos, d, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
            });
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetT(Q<T>& _q, Fv _tembc, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) {
                gpu::record_bc(_q, 1, PL_BC_AD_T, a, pos, d, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _tembc);
            });
        }

        //  BoundaryConditionSetQ (advection.h:241-524, 1093-1130): heat flux, constant diffusivity
        //  (PL_BC_AD_QC, kappa = _diffusivity) or per-node diffusivity (PL_BC_AD_Q)
        namespace detail {
            template<class T, template<class>class Q, class Fv, class Ff>
            void setq(Q<T>& _q, int _a, int _pos, int _d, const Fv &_qnbc, const T *_ux, T _diffusivity, const Ff &_bctype) {
                gpu::record_bc(_q, 1, PL_BC_AD_QC, _a, _pos, _d, _bctype, gpu::IN_FORWARD, _ux, 0.0, double(_diffusivity), _qnbc);
            }
            template<class T, template<class>class Q, class Fv, class Ff>
            void setq(Q<T>& _q, int _a, int _pos, int _d, const Fv &_qnbc, const T *_ux, const T *_diffusivity, const Ff &_bctype) {
                gpu::own(_q, 1).input(PL_KAPPA, _diffusivity);
                gpu::record_bc(_q, 1, PL_BC_AD_Q, _a, _pos, _d, _bctype, gpu::IN_FORWARD, _ux, 0.0, 0.0, _qnbc);
            }
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongXEdge(Q<T>& _q, int _i, int _directionx, Fv _qnbc, const T *_ux, const T *_uy, T _diffusivity, Ff _bctype) { detail::setq(_q, 0, _i, _directionx, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongYEdge(Q<T>& _q, int _j, int _directiony, Fv _qnbc, const T *_ux, const T *_uy, T _diffusivity, Ff _bctype) { detail::setq(_q, 1, _j, _directiony, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongXFace(Q<T>& _q, int _i, int _directionx, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, T _diffusivity, Ff _bctype) { detail::setq(_q, 0, _i, _directionx, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongYFace(Q<T>& _q, int _j, int _directiony, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, T _diffusivity, Ff _bctype) { detail::setq(_q, 1, _j, _directiony, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongZFace(Q<T>& _q, int _k, int _directionz, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, T _diffusivity, Ff _bctype) { detail::setq(_q, 2, _k, _directionz, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongXEdge(Q<T>& _q, int _i, int _directionx, Fv _qnbc, const T *_ux, const T *_uy, const T *_diffusivity, Ff _bctype) { detail::setq(_q, 0, _i, _directionx, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongYEdge(Q<T>& _q, int _j, int _directiony, Fv _qnbc, const T *_ux, const T *_uy, const T *_diffusivity, Ff _bctype) { detail::setq(_q, 1, _j, _directiony, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongXFace(Q<T>& _q, int _i, int _directionx, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, const T *_diffusivity, Ff _bctype) { detail::setq(_q, 0, _i, _directionx, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongYFace(Q<T>& _q, int _j, int _directiony, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, const T *_diffusivity, Ff _bctype) { detail::setq(_q, 1, _j, _directiony, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQAlongZFace(Q<T>& _q, int _k, int _directionz, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, const T *_diffusivity, Ff _bctype) { detail::setq(_q, 2, _k, _directionz, _qnbc, _ux, _diffusivity, _bctype); }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQ(Q<T>& _q, Fv _qnbc, const T *_ux, const T *_uy, T _diffusivity, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::setq(_q, a, pos, d, _qnbc, _ux, _diffusivity, _bctype); });
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQ(Q<T>& _q, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, T _diffusivity, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::setq(_q, a, pos, d, _qnbc, _ux, _diffusivity, _bctype); });
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQ(Q<T>& _q, Fv _qnbc, const T *_ux, const T *_uy, const T *_diffusivity, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::setq(_q, a, pos, d, _qnbc, _ux, _diffusivity, _bctype); });
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void BoundaryConditionSetQ(Q<T>& _q, Fv _qnbc, const T *_ux, const T *_uy, const T *_uz, const T *_diffusivity, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::setq(_q, a, pos, d, _qnbc, _ux, _diffusivity, _bctype); });
        }
    }
}
