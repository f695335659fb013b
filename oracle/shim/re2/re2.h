// Test infrastructure (oracle only): a std::regex stand-in for the RE2 calls in
// the reference's include/statement.h:120-160 (LIKE filters).  Those filters run
// outside Contest::execute, so the join path never reaches this code; it only
// has to compile.  Nothing in the shipped library includes it.
#pragma once
#include <regex>
#include <string>
#include <string_view>

class RE2 {
public:
    struct Options {};
    RE2(const std::string& pattern, const Options&) {
        try {
            re_ = std::regex(pattern);
            ok_ = true;
        } catch (const std::regex_error&) {
            ok_ = false;
        }
    }
    bool ok() const { return ok_; }
    static bool FullMatch(std::string_view s, const RE2& re) {
        return re.ok_ && std::regex_match(s.begin(), s.end(), re.re_);
    }

private:
    std::regex re_;
    bool       ok_ = false;
};
