//  normalize.h -- drop-in Normalize (utility/normalize.h:8-23 of the reference): v /= max |v|,
//  reduced and scaled on the device of a live lattice.
#pragma once
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    template<class T>
    void Normalize(T *_v, int _size) {
        for (gpu::Pair *pr : gpu::live_pairs()) {
            if ((long long)_size > (long long)pr->n * pr->q) continue;   // the library's staging bound
            std::vector<double> v(_v, _v + _size);
            gpu::ck(pl_normalize(pr->h, v.data(), _size), "pl_normalize");
            gpu::to_host(_v, v);
            return;
        }
        gpu::die("Normalize: no lattice on the device is large enough to stage this array");
    }
}
