// Test infrastructure: out-of-line members of the Point2<int> specialization
// declared in oracle/shim/geometry_prelude.h (see there for why it exists).
#include "src/geometry.h"

namespace turner {

Point2<int>::Point2(int x_, int y_) : x(x_), y(y_) {}
int Point2<int>::operator[](Axis2 ax) const { return ax == Axis2::X ? x : y; }
int& Point2<int>::operator[](Axis2 ax) { return ax == Axis2::X ? x : y; }
int Point2<int>::operator[](size_t i) const { return i == 0 ? x : y; }
int& Point2<int>::operator[](size_t i) { return i == 0 ? x : y; }
bool Point2<int>::operator==(const Point2<int>& p) const { return x == p.x && y == p.y; }
bool Point2<int>::operator!=(const Point2<int>& p) const { return !(*this == p); }
Vector2<int> Point2<int>::operator-(const Point2<int>& p) const { return {x - p.x, y - p.y}; }
std::string Point2<int>::to_string() const { return "(" + std::to_string(x) + ", " + std::to_string(y) + ")"; }

} // namespace turner
