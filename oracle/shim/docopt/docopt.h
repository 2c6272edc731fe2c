// Test-infrastructure shim: config.h names docopt::value in its from_docopt()
// parsers. The oracle fills TracerConfig directly and never parses argv.
#pragma once

#include <string>

namespace docopt {
struct value {
    bool asBool() const { return false; }
    long asLong() const { return 0; }
    std::string asString() const { return {}; }
    explicit operator bool() const { return false; }
};
} // namespace docopt
