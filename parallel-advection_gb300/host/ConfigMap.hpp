// INI runtime parameters with the reference's parsing rules (ConfigMap over
// inih: src/config/ConfigMap.cpp:35-92, src/config/inih/ini.cpp:30-140):
//  - "[section]" lines; "name = value" pairs; keys are case-insensitive
//    ("section.name" lower-cased);
//  - ';' or '#' at the start of a line is a comment; an inline comment needs
//    ';' preceded by whitespace ('#' inside a value is kept);
//  - a non-blank line starting with whitespace continues the previous name and
//    replaces its value;
//  - getInteger parses with strtol(base 0) (decimal, 0x hex, 0 octal) and
//    falls back to the default when nothing parses;
//  - getFloat parses with strtof, i.e. every real is rounded to float before it
//    is widened to double (dt = 0.001 becomes 0.0010000000474974513);
//  - getBool accepts 1/yes/true/on and 0/no/false/off, default otherwise.
#pragma once
#include <map>
#include <string>

namespace bkma_host {

class ConfigMap {
  public:
    explicit ConfigMap(const std::string &filename);
    // 0 on success, -1 if the file cannot be opened, else the first bad line
    int parseError() const { return error_; }
    std::string getString(const std::string &section, const std::string &name,
                          const std::string &default_value) const;
    long getInteger(const std::string &section, const std::string &name, long default_value) const;
    double getFloat(const std::string &section, const std::string &name, float default_value) const;
    bool getBool(const std::string &section, const std::string &name, bool default_value) const;

  private:
    std::map<std::string, std::string> values_;
    int error_ = 0;
};

}  // namespace bkma_host
