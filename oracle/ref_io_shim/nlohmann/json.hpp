/* Stand-in for <nlohmann/json.hpp>: libmat's io_utils.hpp includes it, uses
 * nothing of it, and relies on the standard headers that it brings in.
 * Test infrastructure only. */
#pragma once
#include <istream>
#include <locale>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
