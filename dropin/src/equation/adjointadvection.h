//  adjointadvection.h -- drop-in AAD (adjoint advection-diffusion) routines
//  (equation/adjointadvection.h of the reference) on the GB300 library. The coupled adjoint
//  collides read the forward solution (_rho, _ux, _uy[, _uz], _tem) and run fused with the
//  recorded iStream and adjoint boundary routines (see ../gpu/runtime.h).
#pragma once
#include <cmath>
#include "adjointnavierstokes.h"

namespace PANSLBM2 {
    namespace AAD {
        namespace detail {
            template<class T, template<class>class P, template<class>class Q>
            void collide(P<T>& _p, Q<T>& _q, int _kind, const pl_phys &_ph, bool _issave,
                         const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem,
                         T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, T *_item, T *_iqx, T *_iqy, T *_iqz,
                         const T *_alpha, const T *_kappa, const T *_beta, const T *_dirx, const T *_diry, const T *_dirz, T *_ig) {
                gpu::Pair &pr = gpu::couple(_p, _q);
                pr.input(PL_ALPHA, _alpha);
                pr.input(PL_KAPPA, _kappa);
                pr.input(PL_BETA, _beta);
                pr.input(PL_DIRX, _dirx);
                pr.input(PL_DIRY, _diry);
                pr.input(PL_DIRZ, _dirz);
                pr.input(PL_FWD_RHO, _rho);
                pr.input(PL_FWD_UX, _ux);
                pr.input(PL_FWD_UY, _uy);
                pr.input(PL_FWD_UZ, _uz);
                pr.input(PL_FWD_TEM, _tem);
                for (int f = PL_FWD_RHO; f <= PL_FWD_TEM; ++f) pr.forward_default(f);
                T *outs[11] = {_ip, _iux, _iuy, _iuz, _imx, _imy, _imz, _item, _iqx, _iqy, _iqz};
                pr.collide(_kind, _ph, _issave, outs, 11, _ig);
            }
        }

        //  MacroBrinkmanCollideHeatExchange (adjointadvection.h:892-993)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideHeatExchange(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, const T *_beta, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AAD_HEATEX, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, (const T *)nullptr, _tem, _ip, _iux, _iuy, (T *)nullptr, _imx, _imy, (T *)nullptr, _item, _iqx, _iqy, (T *)nullptr,
                            _alpha, (const T *)nullptr, _beta, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideHeatExchange(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz, T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, T *_iqz, const T *_beta, T _diffusivity, bool _issave = false) {
            detail::collide(_p, _q, PL_AAD_HEATEX, gpu::phys<T>(_viscosity, _diffusivity, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _ip, _iux, _iuy, _iuz, _imx, _imy, _imz, _item, _iqx, _iqy, _iqz,
                            _alpha, (const T *)nullptr, _beta, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (T *)nullptr);
        }

        //  MacroBrinkmanCollideForceConvection (adjointadvection.h:995-1109)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideForceConvection(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, const T *_diffusivity, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_FORCE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, (const T *)nullptr, _tem, _ip, _iux, _iuy, (T *)nullptr, _imx, _imy, (T *)nullptr, _item, _iqx, _iqy, (T *)nullptr,
                            _alpha, _diffusivity, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, _ig);
        }
        //  (the reference's 3D routine does not store iuz; the caller's _iuz keeps its values)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideForceConvection(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz, T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, T *_iqz, const T *_diffusivity, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_FORCE, gpu::phys<T>(_viscosity, 0, 0, 0, 0, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _ip, _iux, _iuy, (T *)nullptr, _imx, _imy, _imz, _item, _iqx, _iqy, _iqz,
                            _alpha, _diffusivity, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, _ig);
        }

        //  MacroBrinkmanCollideNaturalConvection (adjointadvection.h:1111-1230): the heat-sink drivers' adjoint collide
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvection(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, const T *_diffusivity, T _gx, T _gy, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_NATURAL, gpu::phys<T>(_viscosity, 0, _gx, _gy, 0, 0), _issave,
                            _rho, _ux, _uy, (const T *)nullptr, _tem, _ip, _iux, _iuy, (T *)nullptr, _imx, _imy, (T *)nullptr, _item, _iqx, _iqy, (T *)nullptr,
                            _alpha, _diffusivity, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, _ig);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvection(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz, T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, T *_iqz, const T *_diffusivity, T _gx, T _gy, T _gz, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_NATURAL, gpu::phys<T>(_viscosity, 0, _gx, _gy, _gz, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _ip, _iux, _iuy, _iuz, _imx, _imy, _imz, _item, _iqx, _iqy, _iqz,
                            _alpha, _diffusivity, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, _ig);
        }

        //  MacroBrinkmanCollideNaturalConvectionMassFlow (adjointadvection.h:1232-1355)
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvectionMassFlow(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, T *_ip, T *_iux, T *_iuy, T *_imx, T *_imy, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, const T *_diffusivity, T _gx, T _gy, const T *_directionx, const T *_directiony, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_MASSFLOW, gpu::phys<T>(_viscosity, 0, _gx, _gy, 0, 0), _issave,
                            _rho, _ux, _uy, (const T *)nullptr, _tem, _ip, _iux, _iuy, (T *)nullptr, _imx, _imy, (T *)nullptr, _item, _iqx, _iqy, (T *)nullptr,
                            _alpha, _diffusivity, (const T *)nullptr, _directionx, _directiony, (const T *)nullptr, _ig);
        }
        template<class T, template<class>class P, template<class>class Q>
        void MacroBrinkmanCollideNaturalConvectionMassFlow(P<T>& _p, const T *_rho, const T *_ux, const T *_uy, const T *_uz, T *_ip, T *_iux, T *_iuy, T *_iuz, T *_imx, T *_imy, T *_imz, const T *_alpha, T _viscosity, Q<T>& _q, const T *_tem, T *_item, T *_iqx, T *_iqy, T *_iqz, const T *_diffusivity, T _gx, T _gy, T _gz, const T *_directionx, const T *_directiony, const T *_directionz, bool _issave = false, T *_ig = nullptr) {
            detail::collide(_p, _q, PL_AAD_MASSFLOW, gpu::phys<T>(_viscosity, 0, _gx, _gy, _gz, 0), _issave,
                            _rho, _ux, _uy, _uz, _tem, _ip, _iux, _iuy, _iuz, _imx, _imy, _imz, _item, _iqx, _iqy, _iqz,
                            _alpha, _diffusivity, (const T *)nullptr, _directionx, _directiony, _directionz, _ig);
        }

        //  InitialCondition (adjointadvection.h:1357-1381)
        template<class T, template<class>class Q>
        void InitialCondition(Q<T>& _q, const T *_ux, const T *_uy, const T *_item, const T *_iqx, const T *_iqy) {
            gpu::Pair &pr = gpu::own(_q, 1);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> x(_ux, pr.n), y(_uy, pr.n), it(_item, pr.n), qx(_iqx, pr.n), qy(_iqy, pr.n);
            std::vector<double> z(pr.n, 0.0);
            gpu::ck(pl_init(pr.h, 3, it.p, qx.p, qy.p, z.data(), x.p, y.p, z.data()), "pl_init");
        }
        template<class T, template<class>class Q>
        void InitialCondition(Q<T>& _q, const T *_ux, const T *_uy, const T *_uz, const T *_item, const T *_iqx, const T *_iqy, const T *_iqz) {
            gpu::Pair &pr = gpu::own(_q, 1);
            pr.flush();
            gpu::sync_outputs();
            gpu::AsDouble<T> x(_ux, pr.n), y(_uy, pr.n), z(_uz, pr.n), it(_item, pr.n), qx(_iqx, pr.n), qy(_iqy, pr.n), qz(_iqz, pr.n);
            gpu::ck(pl_init(pr.h, 3, it.p, qx.p, qy.p, qz.p, x.p, y.p, z.p), "pl_init");
        }

        //  iBoundaryConditionSetT (adjointadvection.h:152-301, 1383-1401); _ux, _uy[, _uz]: the forward velocity
        namespace detail {
            template<class T, template<class>class Q, class Ff>
            void isett(Q<T>& _q, int _a, int _pos, int _d, const T *_ux, const T *_uy, const T *_uz, const Ff &_bctype) {
                gpu::Pair &pr = gpu::own(_q, 1);
                pr.input(PL_FWD_UX, _ux);
                pr.input(PL_FWD_UY, _uy);
                pr.input(PL_FWD_UZ, _uz);
                gpu::record_bc(_q, 1, PL_BC_AAD_T, _a, _pos, _d, _bctype, gpu::IN_ADJOINT);
            }
            template<class T, template<class>class Q, class Ff>
            void isetq(Q<T>& _q, int _a, int _pos, int _d, const T *_ux, const T *_uy, const T *_uz, const Ff &_bctype, T _eps) {
                gpu::Pair &pr = gpu::own(_q, 1);
                pr.input(PL_FWD_UX, _ux);
                pr.input(PL_FWD_UY, _uy);
                pr.input(PL_FWD_UZ, _uz);
                gpu::record_bc(_q, 1, PL_BC_AAD_Q, _a, _pos, _d, _bctype, gpu::IN_ADJOINT, nullptr, double(_eps));
            }
            template<class T, template<class>class P, template<class>class Q, class Ff>
            void isetrho(P<T>& _p, Q<T>& _q, int _a, int _pos, int _d, const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem, const Ff &_bctype, T _eps) {
                gpu::Pair &pr = gpu::couple(_p, _q);
                pr.input(PL_FWD_RHO, _rho);
                pr.input(PL_FWD_UX, _ux);
                pr.input(PL_FWD_UY, _uy);
                pr.input(PL_FWD_UZ, _uz);
                pr.input(PL_FWD_TEM, _tem);
                constexpr int ND = P<T>::nd;
                gpu::Evaluated<int> et = gpu::evaluate<int>(_bctype, "t", _a, _pos, pr.nx, pr.ny, pr.nz,
                                                            [&](int i, int j, int k) { return int(gpu::at<ND>(_bctype, i, j, k)); });
                gpu::BcRec r = gpu::make_rec(PL_BC_AAD_RHO, 0, _a, _pos, _d, &et);
                gpu::finish_rec(r, 3, gpu::IN_ADJOINT, double(_eps));
                pr.record(std::move(r));
            }
        }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetTAlongXEdge(Q<T>& _q, int _i, int _directionx, const T *_ux, const T *_uy, Ff _bctype) { detail::isett(_q, 0, _i, _directionx, _ux, _uy, (const T *)nullptr, _bctype); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetTAlongYEdge(Q<T>& _q, int _j, int _directiony, const T *_ux, const T *_uy, Ff _bctype) { detail::isett(_q, 1, _j, _directiony, _ux, _uy, (const T *)nullptr, _bctype); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetTAlongXFace(Q<T>& _q, int _i, int _directionx, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) { detail::isett(_q, 0, _i, _directionx, _ux, _uy, _uz, _bctype); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetTAlongYFace(Q<T>& _q, int _j, int _directiony, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) { detail::isett(_q, 1, _j, _directiony, _ux, _uy, _uz, _bctype); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetTAlongZFace(Q<T>& _q, int _k, int _directionz, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) { detail::isett(_q, 2, _k, _directionz, _ux, _uy, _uz, _bctype); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetT(Q<T>& _q, const T *_ux, const T *_uy, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::isett(_q, a, pos, d, _ux, _uy, (const T *)nullptr, _bctype); });
        }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetT(Q<T>& _q, const T *_ux, const T *_uy, const T *_uz, Ff _bctype) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::isett(_q, a, pos, d, _ux, _uy, _uz, _bctype); });
        }

        //  iBoundaryConditionSetQ (adjointadvection.h:302-486, 1403-1421): _eps = objective source
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQAlongXEdge(Q<T>& _q, int _i, int _directionx, const T *_ux, const T *_uy, Ff _bctype, T _eps = T()) { detail::isetq(_q, 0, _i, _directionx, _ux, _uy, (const T *)nullptr, _bctype, _eps); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQAlongYEdge(Q<T>& _q, int _j, int _directiony, const T *_ux, const T *_uy, Ff _bctype, T _eps = T()) { detail::isetq(_q, 1, _j, _directiony, _ux, _uy, (const T *)nullptr, _bctype, _eps); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQAlongXFace(Q<T>& _q, int _i, int _directionx, const T *_ux, const T *_uy, const T *_uz, Ff _bctype, T _eps = T()) { detail::isetq(_q, 0, _i, _directionx, _ux, _uy, _uz, _bctype, _eps); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQAlongYFace(Q<T>& _q, int _j, int _directiony, const T *_ux, const T *_uy, const T *_uz, Ff _bctype, T _eps = T()) { detail::isetq(_q, 1, _j, _directiony, _ux, _uy, _uz, _bctype, _eps); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQAlongZFace(Q<T>& _q, int _k, int _directionz, const T *_ux, const T *_uy, const T *_uz, Ff _bctype, T _eps = T()) { detail::isetq(_q, 2, _k, _directionz, _ux, _uy, _uz, _bctype, _eps); }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQ(Q<T>& _q, const T *_ux, const T *_uy, Ff _bctype, T _eps = T()) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::isetq(_q, a, pos, d, _ux, _uy, (const T *)nullptr, _bctype, _eps); });
        }
        template<class T, template<class>class Q, class Ff>
        void iBoundaryConditionSetQ(Q<T>& _q, const T *_ux, const T *_uy, const T *_uz, Ff _bctype, T _eps = T()) {
            gpu::each_face(_q, [&](int a, int pos, int d) { detail::isetq(_q, a, pos, d, _ux, _uy, _uz, _bctype, _eps); });
        }

        //  iBoundaryConditionSetRho (adjointadvection.h:487-751, 1423-1441): type 1 SetT, 2 SetQ
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRhoAlongXEdge(P<T>& _p, Q<T>& _q, int _i, int _directionx, const T *_rho, const T *_ux, const T *_uy, const T *_tem, Ff _bctype, T _eps = T()) { detail::isetrho(_p, _q, 0, _i, _directionx, _rho, _ux, _uy, (const T *)nullptr, _tem, _bctype, _eps); }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRhoAlongYEdge(P<T>& _p, Q<T>& _q, int _j, int _directiony, const T *_rho, const T *_ux, const T *_uy, const T *_tem, Ff _bctype, T _eps = T()) { detail::isetrho(_p, _q, 1, _j, _directiony, _rho, _ux, _uy, (const T *)nullptr, _tem, _bctype, _eps); }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRhoAlongXFace(P<T>& _p, Q<T>& _q, int _i, int _directionx, const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem, Ff _bctypeg, T _eps = T()) { detail::isetrho(_p, _q, 0, _i, _directionx, _rho, _ux, _uy, _uz, _tem, _bctypeg, _eps); }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRhoAlongYFace(P<T>& _p, Q<T>& _q, int _j, int _directiony, const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem, Ff _bctypeg, T _eps = T()) { detail::isetrho(_p, _q, 1, _j, _directiony, _rho, _ux, _uy, _uz, _tem, _bctypeg, _eps); }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRhoAlongZFace(P<T>& _p, Q<T>& _q, int _k, int _directionz, const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem, Ff _bctypeg, T _eps = T()) { detail::isetrho(_p, _q, 2, _k, _directionz, _rho, _ux, _uy, _uz, _tem, _bctypeg, _eps); }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRho(P<T>& _p, Q<T>& _q, const T *_rho, const T *_ux, const T *_uy, const T *_tem, Ff _bctype, T _eps = T()) {
            gpu::each_face(_p, [&](int a, int pos, int d) { detail::isetrho(_p, _q, a, pos, d, _rho, _ux, _uy, (const T *)nullptr, _tem, _bctype, _eps); });
        }
        template<class T, template<class>class P, template<class>class Q, class Ff>
        void iBoundaryConditionSetRho(P<T>& _p, Q<T>& _q, const T *_rho, const T *_ux, const T *_uy, const T *_uz, const T *_tem, Ff _bctypeg, T _eps = T()) {
            gpu::each_face(_p, [&](int a, int pos, int d) { detail::isetrho(_p, _q, a, pos, d, _rho, _ux, _uy, _uz, _tem, _bctypeg, _eps); });
        }

        //  SensitivityHeatExchange (adjointadvection.h:1443-1457)
        template<class T, template<class>class Q>
        void SensitivityHeatExchange(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_imx, const T *_imy, const T *_dads, const T *_tem, const T *_item, const T *_dbds) {
            gpu::sensitivity(gpu::own(_q, 1), 2, _dfds, _dads, _dbds, _ux, _uy, (const T *)nullptr, _tem, _imx, _imy, (const T *)nullptr,
                             _item, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr,
                             (const double *)nullptr, (const int *)nullptr);
        }
        template<class T, template<class>class Q>
        void SensitivityHeatExchange(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_uz, const T *_imx, const T *_imy, const T *_imz, const T *_dads, const T *_tem, const T *_item, const T *_dbds) {
            gpu::sensitivity(gpu::own(_q, 1), 2, _dfds, _dads, _dbds, _ux, _uy, _uz, _tem, _imx, _imy, _imz,
                             _item, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr,
                             (const double *)nullptr, (const int *)nullptr);
        }

        //  SensitivityBrinkmanDiffusivity (adjointadvection.h:1459-1493)
        template<class T, template<class>class Q>
        void SensitivityBrinkmanDiffusivity(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_imx, const T *_imy, const T *_dads, const T *_tem, const T *_item, const T *_iqx, const T *_iqy, const T *_g, const T *_ig, const T *_diffusivity, const T *_dkds) {
            gpu::sensitivity(gpu::own(_q, 1), 1, _dfds, _dads, _dkds, _ux, _uy, (const T *)nullptr, _tem, _imx, _imy, (const T *)nullptr,
                             _item, _iqx, _iqy, (const T *)nullptr, _diffusivity, _g, _ig, (const double *)nullptr, (const int *)nullptr);
        }
        template<class T, template<class>class Q>
        void SensitivityBrinkmanDiffusivity(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_uz, const T *_imx, const T *_imy, const T *_imz, const T *_dads, const T *_tem, const T *_item, const T *_iqx, const T *_iqy, const T *_iqz, const T *_g, const T *_ig, const T *_diffusivity, const T *_dkds) {
            gpu::sensitivity(gpu::own(_q, 1), 1, _dfds, _dads, _dkds, _ux, _uy, _uz, _tem, _imx, _imy, _imz,
                             _item, _iqx, _iqy, _iqz, _diffusivity, _g, _ig, (const double *)nullptr, (const int *)nullptr);
        }

        //  SensitivityTemperatureAtHeatSource (adjointadvection.h:1495-1543; 3D in the argument
        //  order of the overload the drivers call, adjointadvection_avx.h:1459-1513)
        template<class T, template<class>class Q, class Fv, class Ff>
        void SensitivityTemperatureAtHeatSource(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_imx, const T *_imy, const T *_dads, const T *_tem, const T *_item, const T *_iqx, const T *_iqy, const T *_g, const T *_ig, const T *_diffusivity, const T *_dkds, Fv _qnbc, Ff _bctype) {
            gpu::Pair &pr = gpu::own(_q, 1);
            std::vector<double> qn;
            std::vector<int> mask;
            gpu::face_values<2>(pr, _qnbc, _bctype, qn, mask);
            gpu::sensitivity(pr, 0, _dfds, _dads, _dkds, _ux, _uy, (const T *)nullptr, _tem, _imx, _imy, (const T *)nullptr,
                             _item, _iqx, _iqy, (const T *)nullptr, _diffusivity, _g, _ig, qn.data(), mask.data());
        }
        template<class T, template<class>class Q, class Fv, class Ff>
        void SensitivityTemperatureAtHeatSource(Q<T>& _q, T *_dfds, const T *_ux, const T *_uy, const T *_uz, const T *_imx, const T *_imy, const T *_imz, const T *_dads, const T *_tem, const T *_item, const T *_iqx, const T *_iqy, const T *_iqz, const T *_g, const T *_ig, const T *_diffusivity, const T *_dkds, Fv _qnbc, Ff _bctype) {
            gpu::Pair &pr = gpu::own(_q, 1);
            std::vector<double> qn;
            std::vector<int> mask;
            gpu::face_values<3>(pr, _qnbc, _bctype, qn, mask);
            gpu::sensitivity(pr, 0, _dfds, _dads, _dkds, _ux, _uy, _uz, _tem, _imx, _imy, _imz,
                             _item, _iqx, _iqy, _iqz, _diffusivity, _g, _ig, qn.data(), mask.data());
        }
    }
}
