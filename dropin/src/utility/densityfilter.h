//  densityfilter.h -- drop-in DensityFilter (utility/densityfilter.h:10-515 of the reference):
//  the weighted average of radius R on the device. The weight functor has the form described in
//  heavisidefilter.h.
#pragma once
#include <vector>
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace DensityFilter {
        template<class T, template<class>class P, class F>
        std::vector<T> GetFilteredValue(P<T>& _p, T _R, const std::vector<T> &_v, F _weight) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            const auto plan = gpu::filter_plan(pr, double(_R), _weight);
            std::vector<double> v(_v.begin(), _v.end()), out(pr.n);
            if (plan->general)
                gpu::ck(pl_filter_weighted(pr.h, 2, double(_R), 0.0, v.data(), nullptr, plan->table.data(), out.data()),
                        "pl_filter_weighted");
            else
                gpu::ck(pl_density_filter(pr.h, double(_R), v.data(), plan->mask.empty() ? nullptr : plan->mask.data(),
                                          out.data()), "pl_density_filter");
            return std::vector<T>(out.begin(), out.end());
        }

        template<class T, template<class>class P>
        std::vector<T> GetFilteredValue(P<T>& _p, T _R, const std::vector<T> &_v) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            std::vector<double> v(_v.begin(), _v.end()), out(pr.n);
            gpu::ck(pl_density_filter(pr.h, double(_R), v.data(), nullptr, out.data()), "pl_density_filter");
            return std::vector<T>(out.begin(), out.end());
        }
    }
}
