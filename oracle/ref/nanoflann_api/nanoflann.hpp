// nanoflann.hpp — the part of the nanoflann 1.8.0 API that AdaptiveSph's StaticBoundaryDomain.cu uses (a 3-D
// KD-tree radius search over a point cloud adaptor), restated for compiling the reference's library as a checker
// (TEST INFRASTRUCTURE ONLY: it builds oracle/_ref). nanoflann is a third-party dependency fetched by the reference's
// CMake (Dependencies.cmake:11-14) and absent here.
//
// What is restated: radiusSearch(query, r2, matches, params) returns every point whose squared L2 distance
// ((dx*dx + dy*dy) + dz*dz, in the adaptor's element type) is below r2, as (index, squared distance) items; sorted by
// distance when params.sorted. The search structure here is a uniform grid of cells of about the search radius,
// built on the first query radius (nanoflann's tree is an acceleration structure: the set found is the same). With
// params.sorted false the items come in cell order, which is not nanoflann's traversal order, so sums over them can
// differ from the reference's in the last bits of float rounding.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <unordered_map>
#include <utility>
#include <vector>

namespace nanoflann {

template <typename IndexType, typename DistanceType>
struct ResultItem {
    IndexType first;
    DistanceType second;
};

struct SearchParameters {
    float eps = 0.0f;
    bool sorted = true;
};

struct KDTreeSingleIndexAdaptorParams {
    KDTreeSingleIndexAdaptorParams(size_t leaf_max_size = 10) : leaf_max_size(leaf_max_size) {}
    size_t leaf_max_size;
};

template <class T, class DataSource, class DistanceType = T, class IndexType = uint32_t>
struct L2_Simple_Adaptor {
    using ElementType = T;
    using DistType = DistanceType;
};

template <class Distance, class DatasetAdaptor, int DIM = -1, class IndexType = uint32_t>
class KDTreeSingleIndexAdaptor {
public:
    using T = typename Distance::ElementType;

    KDTreeSingleIndexAdaptor(int dims, const DatasetAdaptor& dataset,
                             const KDTreeSingleIndexAdaptorParams& = KDTreeSingleIndexAdaptorParams())
        : dims_(dims), data_(dataset) {}

    template <class Result>
    size_t radiusSearch(const T* q, T r2, std::vector<Result>& out, const SearchParameters& p = {}) const {
        build(r2);
        out.clear();
        const size_t n = data_.kdtree_get_point_count();
        if (n == 0) return 0;
        long c[3];
        for (int a = 0; a < 3; a++) c[a] = cell_of(q[a], a);
        for (long z = c[2] - 1; z <= c[2] + 1; z++)
            for (long y = c[1] - 1; y <= c[1] + 1; y++)
                for (long x = c[0] - 1; x <= c[0] + 1; x++) {
                    auto it = cells_.find(key(x, y, z));
                    if (it == cells_.end()) continue;
                    for (uint32_t i : it->second) {
                        const T dx = data_.kdtree_get_pt(i, 0) - q[0];
                        const T dy = data_.kdtree_get_pt(i, 1) - q[1];
                        const T dz = data_.kdtree_get_pt(i, 2) - q[2];
                        const T d2 = (dx * dx + dy * dy) + dz * dz;
                        if (d2 < r2) out.push_back(Result{static_cast<IndexType>(i), d2});
                    }
                }
        if (p.sorted)
            std::sort(out.begin(), out.end(), [](const Result& a, const Result& b) {
                return a.second < b.second || (a.second == b.second && a.first < b.first);
            });
        return out.size();
    }

private:
    long cell_of(T v, int a) const { return (long)std::floor((double)(v - lo_[a]) / (double)cell_); }
    static uint64_t key(long x, long y, long z) {
        return ((uint64_t)(uint32_t)(x + (1 << 20)) << 42) ^ ((uint64_t)(uint32_t)(y + (1 << 20)) << 21) ^
               (uint64_t)(uint32_t)(z + (1 << 20));
    }
    void build(T r2) const {
        std::lock_guard<std::mutex> g(m_);
        if (built_) return;
        const size_t n = data_.kdtree_get_point_count();
        cell_ = std::sqrt((double)r2) * 1.0001 + 1e-12;
        for (int a = 0; a < 3; a++) lo_[a] = n ? data_.kdtree_get_pt(0, a) : T(0);
        for (size_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) lo_[a] = std::min(lo_[a], data_.kdtree_get_pt(i, a));
        for (size_t i = 0; i < n; i++)
            cells_[key(cell_of(data_.kdtree_get_pt(i, 0), 0), cell_of(data_.kdtree_get_pt(i, 1), 1),
                       cell_of(data_.kdtree_get_pt(i, 2), 2))]
                .push_back((uint32_t)i);
        built_ = true;
    }

    int dims_;
    const DatasetAdaptor& data_;
    mutable std::mutex m_;
    mutable bool built_ = false;
    mutable double cell_ = 1.0;
    mutable T lo_[3] = {T(0), T(0), T(0)};
    mutable std::unordered_map<uint64_t, std::vector<uint32_t>> cells_;
};

}  // namespace nanoflann
