// Stand-in for the part of nlohmann::json the reference's reconstruction
// sources, include/MutoConfig.h and MuToTest.cpp use (at, value with a typed
// default, operator[], find/end, dump, stream input, out_of_range, implicit
// conversion to numbers, strings and vectors of them), over this project's
// own JSON reader.  TEST INFRASTRUCTURE ONLY.
#pragma once

#include <istream>
#include <iterator>
#include <string>
#include <vector>

#include "../../../muontomography_gb300/csrc/json.hpp"

namespace nlohmann {

class json {
public:
    typedef muto::json::out_of_range out_of_range;
    typedef json value_type;
    struct iter {
        bool found;
        bool operator!=(const iter& o) const { return found != o.found; }
        bool operator==(const iter& o) const { return found == o.found; }
    };
    json() {}
    json(const muto::json& v) : v_(v) {}
    static json parse(const std::string& s) { return json(muto::json::parse(s)); }
    json at(const std::string& k) const { return json(v_.at(k)); }
    json operator[](const std::string& k) const { return json(v_[k]); }
    json operator[](const char* k) const { return json(v_[std::string(k)]); }
    iter find(const std::string& k) const { return iter{v_.contains(k)}; }
    iter end() const { return iter{false}; }
    std::string dump() const { return v_.dump(); }
    int value(const std::string& k, int d) const { return v_.value(k, d); }
    double value(const std::string& k, double d) const { return v_.value(k, d); }
    bool value(const std::string& k, bool d) const { return v_.value(k, d); }
    std::string value(const std::string& k, const char* d) const { return v_.value(k, d); }
    // implicit conversions, as MuToTest.cpp:26-28,47,78 use them
    operator int() const { return static_cast<int>(v_.get_int()); }
    operator unsigned int() const { return static_cast<unsigned int>(v_.get_int()); }
    operator double() const { return v_.get_double(); }
    operator std::string() const { return v_.get_string(); }
    operator std::vector<std::string>() const {
        std::vector<std::string> o;
        for (const auto& e : v_.items()) o.push_back(e.get_string());
        return o;
    }
    operator std::vector<double>() const {
        std::vector<double> o;
        for (const auto& e : v_.items()) o.push_back(e.get_double());
        return o;
    }
    friend std::istream& operator>>(std::istream& in, json& j) {
        std::string s((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        j.v_ = muto::json::parse(s);
        return in;
    }

private:
    muto::json v_;
};

}  // namespace nlohmann
