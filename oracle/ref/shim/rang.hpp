// Project-written stand-in for the terminal-colour enums the reference names (include/goofit/Color.h);
// streaming one writes nothing.  rang is an empty submodule of the reference.
#pragma once
#include <ostream>

namespace rang {
enum class fg { black = 30, red, green, yellow, blue, magenta, cyan, gray, reset = 39 };
enum class bg { black = 40, red, green, yellow, blue, magenta, cyan, gray, reset = 49 };
enum class style { reset = 0, bold = 1, dim = 2, italic = 3, underline = 4, blink = 5, rblink = 6, reversed = 7,
                   conceal = 8, crossed = 9 };
inline std::ostream &operator<<(std::ostream &os, fg) { return os; }
inline std::ostream &operator<<(std::ostream &os, bg) { return os; }
inline std::ostream &operator<<(std::ostream &os, style) { return os; }
} // namespace rang
