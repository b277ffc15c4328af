// render::Settings handling (host side).
#pragma once

#include "path_gb300.h"

#include <string>

namespace pg {

void default_settings(path_settings &s);
bool settings_from_yaml_text(const std::string &text, path_settings &s,
                             std::string &err);
bool settings_from_yaml_file(const std::string &path, path_settings &s,
                             std::string &err);

} // namespace pg
