// Minimal stand-in for boost::tokenizer<boost::escaped_list_separator<char>>,
// the only Boost facility the reference uses (colocationFinder.cpp:156-192):
// fields separated by ',', '"' quotes, '\\' escapes.  TEST INFRASTRUCTURE.
#pragma once
#include <string>
#include <vector>

namespace boost {
template <class Char = char>
struct escaped_list_separator {};

template <class Sep = escaped_list_separator<char>>
class tokenizer {
public:
    explicit tokenizer(const std::string& s) {
        std::string cur;
        bool inq = false;
        for (size_t i = 0; i < s.size(); ++i) {
            char c = s[i];
            if (c == '\\' && i + 1 < s.size()) {
                char n = s[++i];
                cur.push_back(n == 'n' ? '\n' : n);
            } else if (c == '"') {
                inq = !inq;
            } else if (c == ',' && !inq) {
                toks_.push_back(cur);
                cur.clear();
            } else {
                cur.push_back(c);
            }
        }
        toks_.push_back(cur);
    }
    std::vector<std::string>::const_iterator begin() const { return toks_.begin(); }
    std::vector<std::string>::const_iterator end() const { return toks_.end(); }

private:
    std::vector<std::string> toks_;
};
}  // namespace boost
