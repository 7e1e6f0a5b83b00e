//  d3q15.h -- drop-in D3Q15 particle: the reference's class interface (particle/d3q15.h:24-254)
//  over a device lattice of the GB300 library. Stream / iStream and the boundary routines are
//  recorded and run fused with the next collide (see ../gpu/runtime.h).
//
//  One device domain: the MPI arguments (PEid, mx, my, mz, and the message-tag offset of
//  Stream / iStream) are accepted for source compatibility and must describe a single domain.
//  f0 / f are host mirrors in the reference's layout, filled by CopyToHost and read back by
//  CopyFromHost (the reference's drivers never touch them).
#pragma once
#include <cassert>

#include "../gpu/runtime.h"

namespace PANSLBM2 {
    template<class T>
    class D3Q15 {
public:
        D3Q15() = delete;
        D3Q15(int _lx, int _ly, int _lz, int _PEid = 0, int _mx = 1, int _my = 1, int _mz = 1) :
            lx(_lx), ly(_ly), lz(_lz), PEid(_PEid), mx(_mx), my(_my), mz(_mz),
            PEx(_PEid%_mx), PEy((_PEid/_mx)%_my), PEz(_PEid/(_mx*_my)),
            nx(_lx), ny(_ly), nz(_lz), nxyz(_lx*_ly*_lz), offsetx(0), offsety(0), offsetz(0)
        {
            assert(0 < _lx && 0 < _ly && 0 < _lz && 0 <= _PEid && 0 < _mx && 0 < _my && 0 < _mz);
            if (_mx != 1 || _my != 1 || _mz != 1 || _PEid != 0) gpu::die("D3Q15: one device domain only (mx = my = mz = 1, PEid = 0)");
            this->f0 = new T[this->nxyz];
            this->f = new T[this->nxyz*(nc - 1)];
            this->gpu.bind(nc, this->nx, this->ny, this->nz);
        }
        D3Q15(const D3Q15<T>& _p) = delete;
        ~D3Q15() {
            delete[] this->f0;
            delete[] this->f;
        }

        int Index(int _i, int _j, int _k) const {
            int i = _i == -1 ? this->nx - 1 : (_i == this->nx ? 0 : _i);
            int j = _j == -1 ? this->ny - 1 : (_j == this->ny ? 0 : _j);
            int k = _k == -1 ? this->nz - 1 : (_k == this->nz ? 0 : _k);
            return i + this->nx*j + this->nx*this->ny*k;
        }
        static int IndexF(int _idx, int _c) { return (nc - 1)*_idx + (_c - 1); }
        int IndexPE(int _i, int _j, int _k) const {
            int i = _i == -1 ? this->mx - 1 : (_i == this->mx ? 0 : _i);
            int j = _j == -1 ? this->my - 1 : (_j == this->my ? 0 : _j);
            int k = _k == -1 ? this->mz - 1 : (_k == this->mz ? 0 : _k);
            return i + this->mx*j + this->mx*this->my*k;
        }
        int IndexBCx(int _j, int _k) const { return _j + this->ny*_k; }
        int IndexBCy(int _k, int _i) const { return _k + this->nz*_i; }
        int IndexBCz(int _i, int _j) const { return _i + this->nx*_j; }

        void Stream(int _offset = 0) { (void)_offset; this->gpu.pair->record_stream(this->gpu.set, 0); }
        void iStream(int _offset = 0) { (void)_offset; this->gpu.pair->record_stream(this->gpu.set, 1); }

        template<class Ff>
        void BoundaryConditionAlongXFace(int _i, int _directionx, Ff _bctype) { this->wall(false, 0, _i, _directionx, _bctype); }
        template<class Ff>
        void BoundaryConditionAlongYFace(int _j, int _directiony, Ff _bctype) { this->wall(false, 1, _j, _directiony, _bctype); }
        template<class Ff>
        void BoundaryConditionAlongZFace(int _k, int _directionz, Ff _bctype) { this->wall(false, 2, _k, _directionz, _bctype); }
        template<class Ff>
        void iBoundaryConditionAlongXFace(int _i, int _directionx, Ff _bctype) { this->wall(true, 0, _i, _directionx, _bctype); }
        template<class Ff>
        void iBoundaryConditionAlongYFace(int _j, int _directiony, Ff _bctype) { this->wall(true, 1, _j, _directiony, _bctype); }
        template<class Ff>
        void iBoundaryConditionAlongZFace(int _k, int _directionz, Ff _bctype) { this->wall(true, 2, _k, _directionz, _bctype); }
        void SmoothCornerAlongYZ(int _j, int _k, int _directiony, int _directionz) { this->line(0, _j, _k, _directiony, _directionz); }
        void SmoothCornerAlongZX(int _k, int _i, int _directionz, int _directionx) { this->line(1, _k, _i, _directionz, _directionx); }
        void SmoothCornerAlongXY(int _i, int _j, int _directionx, int _directiony) { this->line(2, _i, _j, _directionx, _directiony); }
        void SmoothCornerAt(int _i, int _j, int _k, int _directionx, int _directiony, int _directionz) {
            gpu::BcRec r = gpu::make_smooth(PL_SMOOTH_AT, this->gpu.set, 0, _i, _j, _k, _directionx, _directiony, _directionz);
            this->gpu.pair->record(std::move(r));
        }

        template<class Ff>
        void BoundaryCondition(Ff _bctype) {
            this->BoundaryConditionAlongXFace(0, -1, _bctype);              //  On xmin
            this->BoundaryConditionAlongXFace(this->lx - 1, 1, _bctype);    //  On xmax
            this->BoundaryConditionAlongYFace(0, -1, _bctype);              //  On ymin
            this->BoundaryConditionAlongYFace(this->ly - 1, 1, _bctype);    //  On ymax
            this->BoundaryConditionAlongZFace(0, -1, _bctype);              //  On zmin
            this->BoundaryConditionAlongZFace(this->lz - 1, 1, _bctype);    //  On zmax
        }
        template<class Ff>
        void iBoundaryCondition(Ff _bctype) {
            this->iBoundaryConditionAlongXFace(0, -1, _bctype);             //  On xmin
            this->iBoundaryConditionAlongXFace(this->lx - 1, 1, _bctype);   //  On xmax
            this->iBoundaryConditionAlongYFace(0, -1, _bctype);             //  On ymin
            this->iBoundaryConditionAlongYFace(this->ly - 1, 1, _bctype);   //  On ymax
            this->iBoundaryConditionAlongZFace(0, -1, _bctype);             //  On zmin
            this->iBoundaryConditionAlongZFace(this->lz - 1, 1, _bctype);   //  On zmax
        }
        //  the reference's whole sequence of corner (and, in 3D, edge-line) smoothings
        //  (particle/d3q15.h:198-220), recorded as one op
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
        static const int nc = 15, nd = 3, cx[nc], cy[nc], cz[nc];
        static const T ei[nc];
        T *f0, *f;

private:
        template<class Ff>
        void wall(bool _adjoint, int _axis, int _pos, int _dir, const Ff &_bctype) {
            auto type = gpu::evaluate<int>(_bctype, "t", _axis, _pos, this->nx, this->ny, this->nz,
                                           [&](int i, int j, int k) { return int(_bctype(i, j, k)); });
            gpu::BcRec r = gpu::make_rec(_adjoint ? PL_BC_IWALL : PL_BC_WALL, this->gpu.set, _axis, _pos, _dir, &type);
            gpu::finish_rec(r, 1 << this->gpu.set, gpu::IN_NONE);
            this->gpu.pair->record(std::move(r));
        }
        void line(int _plane, int _a, int _b, int _da, int _db) {
            gpu::BcRec r = gpu::make_smooth(PL_SMOOTH_LINE, this->gpu.set, _plane, _a, _b, 0, _da, _db, 0);
            this->gpu.pair->record(std::move(r));
        }

        gpu::Particle<T> gpu;
    };

    //  velocity set in the reference's order (particle/d3q15.h:251-254)
    template<class T>const int D3Q15<T>::cx[D3Q15<T>::nc] = { 0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1 };
    template<class T>const int D3Q15<T>::cy[D3Q15<T>::nc] = { 0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1 };
    template<class T>const int D3Q15<T>::cz[D3Q15<T>::nc] = { 0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1 };
    template<class T>const T D3Q15<T>::ei[D3Q15<T>::nc] = { 2.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/9.0, 1.0/72.0, 1.0/72.0, 1.0/72.0, 1.0/72.0, 1.0/72.0, 1.0/72.0, 1.0/72.0, 1.0/72.0 };
}
