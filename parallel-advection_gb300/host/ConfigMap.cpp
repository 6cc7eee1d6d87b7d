#include "ConfigMap.hpp"

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>

namespace bkma_host {
namespace {

std::string lower(std::string s) {
    for (char &c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

std::string rstrip(const std::string &s) {
    size_t e = s.size();
    while (e > 0 && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(0, e);
}

size_t lskip(const std::string &s, size_t i) {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    return i;
}

// Position of `c`, or of a ';' that follows whitespace, or npos.
size_t find_char_or_comment(const std::string &s, size_t from, char c) {
    bool was_space = false;
    for (size_t i = from; i < s.size(); ++i) {
        if (s[i] == c) return i;
        if (was_space && s[i] == ';') return i;
        was_space = std::isspace((unsigned char)s[i]) != 0;
    }
    return std::string::npos;
}

}  // namespace

ConfigMap::ConfigMap(const std::string &filename) {
    std::ifstream in(filename);
    if (!in) {
        error_ = -1;
        return;
    }
    std::string line, section, prev_name;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        if (!line.empty() && line.back() == '\r') line.pop_back();
        const std::string stripped = rstrip(line);
        const size_t start = lskip(stripped, 0);
        if (start >= stripped.size()) continue;  // blank
        const std::string body = stripped.substr(start);
        if (!prev_name.empty() && start > 0) {
            // continuation line: handler called again, value replaced
            values_[lower(section + "." + prev_name)] = body;
            continue;
        }
        if (body[0] == ';' || body[0] == '#') continue;
        if (body[0] == '[') {
            const size_t end = find_char_or_comment(body, 1, ']');
            if (end != std::string::npos && body[end] == ']') {
                section = body.substr(1, end - 1);
                prev_name.clear();
            } else if (!error_) {
                error_ = lineno;
            }
            continue;
        }
        const size_t eq = find_char_or_comment(body, 0, '=');
        if (eq == std::string::npos || body[eq] != '=') {
            if (!error_) error_ = lineno;
            continue;
        }
        const std::string name = rstrip(body.substr(0, eq));
        std::string value = body.substr(lskip(body, eq + 1));
        const size_t cmt = find_char_or_comment(value, 0, '\0');
        if (cmt != std::string::npos && value[cmt] == ';') value = value.substr(0, cmt);
        value = rstrip(value);
        prev_name = name;
        values_[lower(section + "." + name)] = value;
    }
}

std::string ConfigMap::getString(const std::string &section, const std::string &name,
                                 const std::string &default_value) const {
    const auto it = values_.find(lower(section + "." + name));
    return it == values_.end() ? default_value : it->second;
}

long ConfigMap::getInteger(const std::string &section, const std::string &name,
                           long default_value) const {
    const std::string v = getString(section, name, "");
    const char *p = v.c_str();
    char *end = nullptr;
    const long n = std::strtol(p, &end, 0);
    return end > p ? n : default_value;
}

double ConfigMap::getFloat(const std::string &section, const std::string &name,
                           float default_value) const {
    const std::string v = getString(section, name, "");
    const char *p = v.c_str();
    char *end = nullptr;
    const float f = std::strtof(p, &end);
    return end > p ? static_cast<double>(f) : static_cast<double>(default_value);
}

bool ConfigMap::getBool(const std::string &section, const std::string &name,
                        bool default_value) const {
    const std::string v = getString(section, name, "");
    bool val = default_value;
    if (v == "1" || v == "yes" || v == "true" || v == "on") val = true;
    if (v == "0" || v == "no" || v == "false" || v == "off") val = false;
    if (v.empty()) val = default_value;
    return val;
}

}  // namespace bkma_host
