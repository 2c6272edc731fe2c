// Test-infrastructure prelude, force-included (-include) when the reference's
// sources are compiled into oracle/_ref.
//
// Why: src/geometry.h defines `friend` function templates inside the class
// templates Point2<T> (geometry.h:413) and Normal3<T> (geometry.h:741) and then
// explicitly instantiates both float and int variants (geometry.h:1117-1132).
// Every instantiation re-defines the same friend template, which GCC 13
// rejects as a redefinition. The int variants are not used by the path
// tracer. Declaring explicit specializations of Point2<int> and Normal3<int>
// before the primary templates are defined means the explicit instantiations
// of those two types "have no effect" ([temp.explicit]), so the reference's
// headers compile unmodified. The members below are the ones Bbox2<int>,
// Bbox2iIterator and Vector3<int> name; they are defined in
// oracle/geometry_prelude.cpp.
#pragma once

#include <cstddef>
#include <string>

namespace turner {

enum class Axis2 : char;
template <typename T> class Vector2;
template <typename T> class Point2;
template <typename T> class Normal3;

template <> class Point2<int> {
public:
    Point2() = default;
    Point2(int x_, int y_);
    int operator[](Axis2 ax) const;
    int& operator[](Axis2 ax);
    int operator[](size_t i) const;
    int& operator[](size_t i);
    bool operator==(const Point2<int>& p) const;
    bool operator!=(const Point2<int>& p) const;
    Vector2<int> operator-(const Point2<int>& p) const;
    std::string to_string() const;

    int x = 0;
    int y = 0;
};

template <> class Normal3<int> {
public:
    int x = 0;
    int y = 0;
    int z = 0;
};

} // namespace turner
