// dxmc/beams/filters/ctaecfilter.hpp -- tube-current modulation along the scan axis,
// CTAECFilter(start, stop, weights) (datacontainer.cpp:53-62, :146) and the organ AEC
// (angular) filter edited at beamsettingsmodel.cpp:349-438.
#pragma once

#include <array>
#include <vector>

namespace dxmc {

class CTAECFilter {
public:
    CTAECFilter() = default;
    CTAECFilter(const std::array<double, 3>& start, const std::array<double, 3>& stop, const std::vector<double>& weights)
    {
        setData(start, stop, weights);
    }
    void setData(const std::array<double, 3>& start, const std::array<double, 3>& stop, const std::vector<double>& weights)
    {
        m_start = start;
        m_stop = stop;
        m_weights = weights;
    }
    bool isEmpty() const { return m_weights.size() < 2; }
    const std::vector<double>& weights() const { return m_weights; }
    const std::array<double, 3>& startPosition() const { return m_start; }
    const std::array<double, 3>& stopPosition() const { return m_stop; }

private:
    std::array<double, 3> m_start { 0, 0, 0 };
    std::array<double, 3> m_stop { 0, 0, 0 };
    std::vector<double> m_weights;
};

class CTOrganAECFilter {
public:
    bool useFilter() const { return m_use; }
    void setUseFilter(bool on) { m_use = on; }
    double startAngleDeg() const { return m_start; }
    void setStartAngleDeg(double a) { m_start = a; }
    double stopAngleDeg() const { return m_stop; }
    void setStopAngleDeg(double a) { m_stop = a; }
    double rampAngleDeg() const { return m_ramp; }
    void setRampAngleDeg(double a) { m_ramp = a < 0 ? 0 : a; }
    double lowWeightFactor() const { return m_low; }
    void setLowWeightFactor(double f) { m_low = f < 0 ? 0 : (f > 1 ? 1 : f); }
    bool compensateOutside() const { return m_compensate; }
    void setCompensateOutside(bool on) { m_compensate = on; }

private:
    bool m_use = false;
    double m_start = 0.0;
    double m_stop = 180.0;
    double m_ramp = 20.0;
    double m_low = 0.6;
    bool m_compensate = true;
};

} // namespace dxmc
