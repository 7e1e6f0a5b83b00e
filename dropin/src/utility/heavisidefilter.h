//  heavisidefilter.h -- drop-in HeavisideFilter (utility/heavisidefilter.h:404-899 of the
//  reference): the density filter of radius R followed by the Heaviside projection (beta,
//  threshold 0.5), and the chain rule of its sensitivity, on the device.
//
//  A weight functor of the reference drivers' form (the hat weight (R - distance) / R,
//  everywhere or between two nodes of a design region with the identity elsewhere) is
//  recognised and its weights are built on the device; any other functor is evaluated on every
//  (node, tap) pair on the host and its table goes to pl_filter_weighted (gpu::filter_plan).
#pragma once
#include <vector>
#include "../gpu/runtime.h"

namespace PANSLBM2 {
    namespace HeavisideFilter {
        template<class T, template<class>class P, class F>
        std::vector<T> GetFilteredVariable(P<T>& _p, T _R, T _beta, const std::vector<T> &_s, F _weight) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            const auto plan = gpu::filter_plan(pr, double(_R), _weight);
            std::vector<double> s(_s.begin(), _s.end()), out(pr.n);
            if (plan->general)
                gpu::ck(pl_filter_weighted(pr.h, 0, double(_R), double(_beta), s.data(), nullptr, plan->table.data(),
                                           out.data()), "pl_filter_weighted");
            else
                gpu::ck(pl_heaviside_var(pr.h, double(_R), double(_beta), s.data(),
                                         plan->mask.empty() ? nullptr : plan->mask.data(), out.data()), "pl_heaviside_var");
            return std::vector<T>(out.begin(), out.end());
        }

        template<class T, template<class>class P>
        std::vector<T> GetFilteredVariable(P<T>& _p, T _R, T _beta, const std::vector<T> &_s) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            std::vector<double> s(_s.begin(), _s.end()), out(pr.n);
            gpu::ck(pl_heaviside_var(pr.h, double(_R), double(_beta), s.data(), nullptr, out.data()), "pl_heaviside_var");
            return std::vector<T>(out.begin(), out.end());
        }

        template<class T, template<class>class P, class F>
        std::vector<T> GetFilteredSensitivity(P<T>& _p, T _R, T _beta, const std::vector<T> &_s, const std::vector<T> &_dfdrho, F _weight) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            const auto plan = gpu::filter_plan(pr, double(_R), _weight);
            std::vector<double> s(_s.begin(), _s.end()), d(_dfdrho.begin(), _dfdrho.end()), out(pr.n);
            if (plan->general)
                gpu::ck(pl_filter_weighted(pr.h, 1, double(_R), double(_beta), s.data(), d.data(), plan->table.data(),
                                           out.data()), "pl_filter_weighted");
            else
                gpu::ck(pl_heaviside_sens(pr.h, double(_R), double(_beta), s.data(), d.data(),
                                          plan->mask.empty() ? nullptr : plan->mask.data(), out.data()), "pl_heaviside_sens");
            return std::vector<T>(out.begin(), out.end());
        }

        template<class T, template<class>class P>
        std::vector<T> GetFilteredSensitivity(P<T>& _p, T _R, T _beta, const std::vector<T> &_s, const std::vector<T> &_dfdrho) {
            gpu::Pair &pr = *_p.gpu_particle().pair;
            gpu::sync_outputs();
            std::vector<double> s(_s.begin(), _s.end()), d(_dfdrho.begin(), _dfdrho.end()), out(pr.n);
            gpu::ck(pl_heaviside_sens(pr.h, double(_R), double(_beta), s.data(), d.data(), nullptr, out.data()), "pl_heaviside_sens");
            return std::vector<T>(out.begin(), out.end());
        }
    }
}
