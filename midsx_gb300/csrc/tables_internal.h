// tables_internal.h - helpers shared by the host sources of libmidsx_gb300.
#pragma once
#include <string>

namespace midsx {
void set_last_error(const std::string& s);
const char* last_error();
}  // namespace midsx
