// dxmc/world/world.hpp -- World<Items...>: owns world items (addItem<T>() returns a
// stable reference) and builds them (simulationpipeline.cpp:127-131, :153).
#pragma once

#include <deque>
#include <tuple>
#include <utility>

namespace dxmc {

template <typename... Items>
class World {
public:
    template <typename U>
    U& addItem()
    {
        return std::get<std::deque<U>>(m_items).emplace_back();
    }

    void build()
    {
        forEachItem([](auto& item) { item.build(); });
    }

    template <typename F>
    void forEachItem(F&& f)
    {
        std::apply([&](auto&... lists) { (forAll(lists, f), ...); }, m_items);
    }

private:
    template <typename L, typename F>
    static void forAll(L& list, F& f)
    {
        for (auto& item : list)
            f(item);
    }

    std::tuple<std::deque<Items>...> m_items;
};

} // namespace dxmc
