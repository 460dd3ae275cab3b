// Compile-only stand-in for the JSON library the reference's save.hpp
// includes (nlohmann/json, not available here).  TEST INFRASTRUCTURE: it lets
// oracle/ref_grid_shim.cpp compile the reference's cube.hpp unchanged for its
// grid evaluation functions; the shim never calls the reference's JSON
// writers, so every operation here is a no-op.
#pragma once
#include <initializer_list>
#include <ostream>
#include <string>

namespace nlohmann {

class ordered_json {
public:
    ordered_json() = default;
    template <typename T>
    ordered_json(const T&) {}
    ordered_json(std::initializer_list<ordered_json>) {}
    template <typename T>
    ordered_json& operator=(const T&) { return *this; }
    template <typename K>
    ordered_json& operator[](const K&) { return *this; }
    std::string dump(int = -1) const { return "{}"; }
    friend std::ostream& operator<<(std::ostream& os, const ordered_json&) { return os; }
};

using json = ordered_json;

}  // namespace nlohmann
