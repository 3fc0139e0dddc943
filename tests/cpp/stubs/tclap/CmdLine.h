// Test stub of the TCLAP command-line parser the reference's examples include: just enough for
// their argument handling to compile and for `-n=<events>` / `--nevents=<events>` to parse.
#pragma once
#include <cstdlib>
#include <string>
#include <vector>

namespace TCLAP {

class ArgException {
public:
    std::string error() const { return "argument error"; }
    std::string argId() const { return "?"; }
};

class ArgBase {
public:
    virtual ~ArgBase() = default;
    virtual void parse(const std::string& a) = 0;
};

template <typename T>
class ValueArg : public ArgBase {
public:
    ValueArg(const std::string& flag, const std::string& name, const std::string&, bool, T dflt, const std::string&)
        : flag_("-" + flag + "="), name_("--" + name + "="), value_(dflt) {}
    T getValue() const { return value_; }
    void parse(const std::string& a) override
    {
        for (const std::string& p : {flag_, name_})
            if (a.compare(0, p.size(), p) == 0) value_ = static_cast<T>(std::strtod(a.c_str() + p.size(), nullptr));
    }

private:
    std::string flag_, name_;
    T value_;
};

class CmdLine {
public:
    CmdLine(const std::string&, char, const std::string& = "") {}
    void add(ArgBase& a) { args_.push_back(&a); }
    void parse(int argc, char** argv)
    {
        for (int i = 1; i < argc; ++i)
            for (ArgBase* a : args_) a->parse(argv[i]);
    }

private:
    std::vector<ArgBase*> args_;
};

}  // namespace TCLAP
