// dxmc/material/nistmaterials.hpp -- named reference materials
// (NISTMaterials::density / Material::byNistName, ctsegmentationpipeline.cpp:73-76).
// The reference's full NIST table is not part of this project; the layer knows
// water, dry air and PMMA (detail::namedComposition).  Unknown names give
// std::nullopt / a density of 0.
#pragma once

#include <map>
#include <optional>
#include <string>
#include <vector>

#include "material.hpp"

namespace dxmc {

class NISTMaterials {
public:
    static std::vector<std::string> listNames()
    {
        return { "Water, Liquid", "Air, Dry (near sea level)", "Polymethyl Methacralate (Lucite, Perspex)" };
    }

    static std::optional<std::map<std::size_t, double>> Composition(const std::string& name)
    {
        return detail::namedComposition(name);
    }

    static double density(const std::string& name)
    {
        if (name == "Water, Liquid")
            return 1.0;
        if (name == "Air, Dry (near sea level)")
            return 0.001205;
        if (name == "Polymethyl Methacralate (Lucite, Perspex)")
            return 1.19;
        return 0.0;
    }
};

} // namespace dxmc
