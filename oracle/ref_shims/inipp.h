// Minimal INI reader with the interface MCAC's PhysicalModel constructor uses
// (physical_model/physical_model.cpp:101-187): Ini<char>{sections, parse,
// interpolate, generate} and extract(). Written for the oracle build of the
// reference only; it is test infrastructure, never part of the product.
//
// Semantics kept from the upstream inipp library the reference links:
//  * "[section]" opens a section, "key = value" lines are trimmed, lines whose
//    first non-blank character is ';' or '#' are comments;
//  * the first definition of a key wins (map emplace);
//  * extract() into a string assigns the value even when it is empty
//    (the reference reuses one string for three keys and relies on that);
//  * extract() into any other type parses with std::boolalpha and leaves the
//    destination unchanged unless the whole value parses.
#ifndef ORACLE_SHIM_INIPP_H
#define ORACLE_SHIM_INIPP_H
#include <istream>
#include <map>
#include <ostream>
#include <sstream>
#include <string>

namespace inipp {

inline std::string trim_copy(const std::string &s) {
    const char *ws = " \t\r\n\f\v";
    size_t b = s.find_first_not_of(ws);
    if (b == std::string::npos) return std::string();
    size_t e = s.find_last_not_of(ws);
    return s.substr(b, e - b + 1);
}

template <class CharT>
class Ini {
  public:
    using String = std::basic_string<CharT>;
    using Section = std::map<String, String>;
    std::map<String, Section> sections;

    void parse(std::basic_istream<CharT> &is) {
        String line;
        String current;
        while (std::getline(is, line)) {
            String t = trim_copy(line);
            if (t.empty() || t[0] == ';' || t[0] == '#') continue;
            if (t[0] == '[') {
                size_t close = t.find(']');
                if (close != String::npos) current = trim_copy(t.substr(1, close - 1));
                continue;
            }
            size_t eq = t.find('=');
            if (eq == String::npos) continue;
            String key = trim_copy(t.substr(0, eq));
            String value = trim_copy(t.substr(eq + 1));
            sections[current].emplace(key, value);
        }
    }
    void interpolate() {}
    void generate(std::basic_ostream<CharT> &os) const {
        for (const auto &sec : sections) {
            os << '[' << sec.first << ']' << '\n';
            for (const auto &kv : sec.second) os << kv.first << " = " << kv.second << '\n';
            os << '\n';
        }
    }
};

template <class CharT, class T>
inline bool extract(const std::basic_string<CharT> &value, T &dst) {
    CharT c;
    std::basic_istringstream<CharT> is{value};
    T result;
    if ((is >> std::boolalpha >> result) && !(is >> c)) {
        dst = result;
        return true;
    }
    return false;
}

template <class CharT>
inline bool extract(const std::basic_string<CharT> &value, std::basic_string<CharT> &dst) {
    dst = value;
    return true;
}

}  // namespace inipp
#endif
