//  d2q9.h -- drop-in D2Q9 particle: the reference's class interface (particle/d2q9.h:24-163)
//  over a device lattice of the GB300 library. Stream / iStream and the boundary routines are
//  recorded and run fused with the next collide (see ../gpu/runtime.h).
//
//  One device domain: the MPI arguments (PEid, mx, my) are accepted for source compatibility
//  and must describe a single domain. f0 / f are host mirrors in the reference's layout, filled
//  by CopyToHost and read back by CopyFromHost (the reference's drivers never touch them).
#pragma once
#include <cassert>

#include "../gpu/runtime.h"

namespace PANSLBM2 {
    template<class T>
    class D2Q9 {
public:
        D2Q9() = delete;
        D2Q9(int _lx, int _ly, int _PEid = 0, int _mx = 1, int _my = 1) :
            lx(_lx), ly(_ly), lz(1), PEid(_PEid), mx(_mx), my(_my), mz(1),
            PEx(_PEid%_mx), PEy(_PEid/_mx), PEz(0),
            nx(_lx), ny(_ly), nz(1), nxyz(_lx*_ly), offsetx(0), offsety(0), offsetz(0)
        {
            assert(0 < _lx && 0 < _ly && 0 <= _PEid && 0 < _mx && 0 < _my);
            if (_mx != 1 || _my != 1 || _PEid != 0) gpu::die("D2Q9: one device domain only (mx = my = 1, PEid = 0)");
            this->f0 = new T[this->nxyz];
            this->f = new T[this->nxyz*(nc - 1)];
            this->gpu.bind(nc, this->nx, this->ny, 1);
        }
        D2Q9(const D2Q9<T>& _p) = delete;
        ~D2Q9() {
            delete[] this->f0;
            delete[] this->f;
        }

        int Index(int _i, int _j) const {
            int i = _i == -1 ? this->nx - 1 : (_i == this->nx ? 0 : _i);
            int j = _j == -1 ? this->ny - 1 : (_j == this->ny ? 0 : _j);
            return i + this->nx*j;
        }
        int Index(int _i, int _j, int _k) const { return this->Index(_i, _j); }
        static int IndexF(int _idx, int _c) { return (nc - 1)*_idx + (_c - 1); }
        int IndexPE(int _i, int _j) const {
            int i = _i == -1 ? this->mx - 1 : (_i == this->mx ? 0 : _i);
            int j = _j == -1 ? this->my - 1 : (_j == this->my ? 0 : _j);
            return i + this->mx*j;
        }
        int IndexPE(int _i, int _j, int _k) const { return this->IndexPE(_i, _j); }

        void Stream() { this->gpu.pair->record_stream(this->gpu.set, 0); }
        void iStream() { this->gpu.pair->record_stream(this->gpu.set, 1); }

        template<class Ff>
        void BoundaryConditionAlongXEdge(int _i, int _directionx, Ff _bctype) { this->wall(false, 0, _i, _directionx, _bctype); }
        template<class Ff>
        void BoundaryConditionAlongYEdge(int _j, int _directiony, Ff _bctype) { this->wall(false, 1, _j, _directiony, _bctype); }
        template<class Ff>
        void iBoundaryConditionAlongXEdge(int _i, int _directionx, Ff _bctype) { this->wall(true, 0, _i, _directionx, _bctype); }
        template<class Ff>
        void iBoundaryConditionAlongYEdge(int _j, int _directiony, Ff _bctype) { this->wall(true, 1, _j, _directiony, _bctype); }
        void SmoothCornerAt(int _i, int _j, int _directionx, int _directiony) {
            gpu::BcRec r = gpu::make_smooth(PL_SMOOTH_AT, this->gpu.set, 0, _i, _j, 0, _directionx, _directiony, 0);
            this->gpu.pair->record(std::move(r));
        }

        template<class Ff>
        void BoundaryCondition(Ff _bctype) {
            this->BoundaryConditionAlongXEdge(0, -1, _bctype);              //  On xmin
            this->BoundaryConditionAlongXEdge(this->lx - 1, 1, _bctype);    //  On xmax
            this->BoundaryConditionAlongYEdge(0, -1, _bctype);              //  On ymin
            this->BoundaryConditionAlongYEdge(this->ly - 1, 1, _bctype);    //  On ymax
        }
        template<class Ff>
        void iBoundaryCondition(Ff _bctype) {
            this->iBoundaryConditionAlongXEdge(0, -1, _bctype);             //  On xmin
            this->iBoundaryConditionAlongXEdge(this->lx - 1, 1, _bctype);   //  On xmax
            this->iBoundaryConditionAlongYEdge(0, -1, _bctype);             //  On ymin
            this->iBoundaryConditionAlongYEdge(this->ly - 1, 1, _bctype);   //  On ymax
        }
        //  the reference's whole sequence of corner (and, in 3D, edge-line) smoothings
        //  (particle/d2q9.h:127-132), recorded as one op
        void SmoothCorner() {
            gpu::BcRec r = gpu::make_smooth(PL_SMOOTH_CORNER, this->gpu.set, 0, 0, 0, 0, 0, 0, 0);
            this->gpu.pair->record(std::move(r));
        }

        //  host mirrors f0 / f (reference layout, f[IndexF(idx, c)]) <-> device populations
        void CopyToHost() {
            gpu::Pair &pr = *this->gpu.pair;
            pr.flush();
            gpu::sync_outputs();
            std::vector<double> p((size_t)nc*this->nxyz);
            gpu::ck(pl_get_populations(pr.h, this->gpu.set, p.data()), "pl_get_populations");
            for (int idx = 0; idx < this->nxyz; ++idx) {
                this->f0[idx] = T(p[idx]);
                for (int c = 1; c < nc; ++c) this->f[IndexF(idx, c)] = T(p[(size_t)c*this->nxyz + idx]);
            }
        }
        void CopyFromHost() {
            gpu::Pair &pr = *this->gpu.pair;
            pr.flush();
            gpu::sync_outputs();
            std::vector<double> p((size_t)nc*this->nxyz);
            for (int idx = 0; idx < this->nxyz; ++idx) {
                p[idx] = double(this->f0[idx]);
                for (int c = 1; c < nc; ++c) p[(size_t)c*this->nxyz + idx] = double(this->f[IndexF(idx, c)]);
            }
            gpu::ck(pl_set_populations(pr.h, this->gpu.set, p.data()), "pl_set_populations");
        }

        gpu::Particle<T> &gpu_particle() { return this->gpu; }

        const int lx, ly, lz, PEid, mx, my, mz, PEx, PEy, PEz, nx, ny, nz, nxyz, offsetx, offsety, offsetz;
        static const int nc = 9, nd = 2, cx[nc], cy[nc], cz[nc];
        static const T ei[nc];
        T *f0, *f;

private:
        template<class Ff>
        void wall(bool _adjoint, int _axis, int _pos, int _dir, const Ff &_bctype) {
            auto type = gpu::evaluate<int>(_bctype, "t", _axis, _pos, this->nx, this->ny, 1,
                                           [&](int i, int j, int) { return int(_bctype(i, j)); });
            gpu::BcRec r = gpu::make_rec(_adjoint ? PL_BC_IWALL : PL_BC_WALL, this->gpu.set, _axis, _pos, _dir, &type);
            gpu::finish_rec(r, 1 << this->gpu.set, gpu::IN_NONE);
            this->gpu.pair->record(std::move(r));
        }

        gpu::Particle<T> gpu;
    };

    //  velocity set in the reference's order (particle/d2q9.h:160-163)
    template<class T>const int D2Q9<T>::cx[D2Q9<T>::nc] = { 0, 1, 0, -1, 0, 1, -1, -1, 1 };
    template<class T>const int D2Q9<T>::cy[D2Q9<T>::nc] = { 0, 0, 1, 0, -1, 1, 1, -1, -1 };
    template<class T>const int D2Q9<T>::cz[D2Q9<T>::nc] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 };
    template<class T>const T D2Q9<T>::ei[D2Q9<T>::nc] = { 4.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0 };
}
