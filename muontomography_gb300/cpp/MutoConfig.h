// JSON configuration (the reference's include/MutoConfig.h:11-46) over this
// project's JSON reader: loadFile, getConfigString, get(key), exist(key).
#pragma once

#include <fstream>
#include <iostream>
#include <iterator>
#include <string>

#include "json.hpp"

using json = muto::json;

class MutoConfig {
public:
    MutoConfig() {}
    explicit MutoConfig(const std::string& filename) {
        if (!loadFile(filename)) std::cerr << "Configuration file load error for: " << filename << std::endl;
    }

    bool loadFile(const std::string& filename) {
        std::ifstream in(filename.c_str());
        if (in.fail()) return false;
        const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        try {
            fConfig = json::parse(text);
        } catch (const std::exception& e) {
            std::cerr << "Configuration file " << filename << ": " << e.what() << std::endl;
            return false;
        }
        return true;
    }
    bool loadString(const std::string& text) {
        try {
            fConfig = json::parse(text);
        } catch (const std::exception&) {
            return false;
        }
        return true;
    }

    std::string getConfigString() const { return fConfig.dump(); }
    // a missing key gives a null value, like nlohmann's operator[]
    const json& get(const std::string& key) const { return fConfig[key]; }
    bool exist(const std::string& key) const { return fConfig.contains(key); }

private:
    json fConfig;
};
