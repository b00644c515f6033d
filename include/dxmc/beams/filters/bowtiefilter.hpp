// dxmc/beams/filters/bowtiefilter.hpp -- relative tube output versus fan angle,
// BowtieFilter(vector<pair<angle_rad, weight>>) as built from the bowtie JSON
// (bowtiefilterreader.cpp:64-92).  Points may come in any order.
#pragma once

#include <algorithm>
#include <utility>
#include <vector>

namespace dxmc {

class BowtieFilter {
public:
    BowtieFilter() = default;
    explicit BowtieFilter(const std::vector<std::pair<double, double>>& angleWeight)
        : m_data(angleWeight)
    {
        std::stable_sort(m_data.begin(), m_data.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    }

    const std::vector<std::pair<double, double>>& data() const { return m_data; }
    bool isEmpty() const { return m_data.empty(); }

    // piecewise-linear weight at |angle|, clamped beyond the table
    double operator()(double angle) const
    {
        if (m_data.empty())
            return 1.0;
        const double a = angle < 0 ? -angle : angle;
        if (a <= m_data.front().first)
            return m_data.front().second;
        if (a >= m_data.back().first)
            return m_data.back().second;
        auto hi = std::upper_bound(m_data.begin(), m_data.end(), a, [](double x, const auto& p) { return x < p.first; });
        auto lo = hi - 1;
        const double t = (a - lo->first) / (hi->first - lo->first);
        return lo->second + t * (hi->second - lo->second);
    }

private:
    std::vector<std::pair<double, double>> m_data;
};

} // namespace dxmc
