// A minimal stand-in for the TCLAP command-line parser, covering only the calls
// canmom/rasteriser's arguments.cpp makes (CmdLine, ValueArg<T>, SwitchArg, parse, getValue,
// ArgException). Where TCLAP is not installed, this lets the reference's own arguments.cpp compile
// unmodified, both for the drop-in link build and for the oracle.
#ifndef RAST_ORACLE_TCLAP_SHIM_H
#define RAST_ORACLE_TCLAP_SHIM_H

#include <cstdlib>
#include <iostream>  // the real TCLAP headers pull in <iostream>; arguments.cpp relies on it
#include <sstream>
#include <string>
#include <vector>

namespace TCLAP {

class ArgException {
public:
    ArgException(const std::string& text, const std::string& id) : text_(text), id_(id) {}
    std::string error() const { return text_; }
    std::string argId() const { return id_; }

private:
    std::string text_, id_;
};

class Arg {
public:
    Arg(const std::string& flag, const std::string& name, bool required, bool takes_value)
        : flag_(flag), name_(name), required_(required), takes_value_(takes_value) {}
    virtual ~Arg() {}
    bool matches(const std::string& token) const {
        return (!flag_.empty() && token == "-" + flag_) || token == "--" + name_;
    }
    bool takes_value() const { return takes_value_; }
    bool required() const { return required_; }
    bool seen() const { return seen_; }
    const std::string& name() const { return name_; }
    virtual void set(const std::string& text) = 0;

protected:
    std::string flag_, name_;
    bool required_, takes_value_;
    bool seen_ = false;
};

class CmdLine {
public:
    CmdLine(const std::string& /*message*/, char /*delimiter*/ = ' ', const std::string& /*version*/ = "none") {}
    void add(Arg* a) { args_.push_back(a); }
    void parse(int argc, char** argv) {
        for (int i = 1; i < argc; ++i) {
            const std::string tok = argv[i];
            Arg* hit = nullptr;
            for (Arg* a : args_)
                if (a->matches(tok)) hit = a;
            if (!hit) throw ArgException("unknown argument", tok);
            if (hit->takes_value()) {
                if (i + 1 >= argc) throw ArgException("missing value", hit->name());
                hit->set(argv[++i]);
            } else {
                hit->set("");
            }
        }
        for (Arg* a : args_)
            if (a->required() && !a->seen()) throw ArgException("required argument missing", a->name());
    }

private:
    std::vector<Arg*> args_;
};

template <typename T>
class ValueArg : public Arg {
public:
    ValueArg(const std::string& flag, const std::string& name, const std::string& /*desc*/, bool req,
             T value, const std::string& /*type_desc*/, CmdLine& cmd)
        : Arg(flag, name, req, true), value_(value) {
        cmd.add(this);
    }
    void set(const std::string& text) override {
        std::istringstream in(text);
        T v;
        if (!(in >> v)) throw ArgException("could not parse value", name_);
        value_ = v;
        seen_ = true;
    }
    T getValue() const { return value_; }

private:
    T value_;
};

template <>
inline void ValueArg<std::string>::set(const std::string& text) {
    value_ = text;
    seen_ = true;
}

class SwitchArg : public Arg {
public:
    SwitchArg(const std::string& flag, const std::string& name, const std::string& /*desc*/, CmdLine& cmd,
              bool def = false)
        : Arg(flag, name, false, false), value_(def) {
        cmd.add(this);
    }
    void set(const std::string&) override { value_ = !value_; seen_ = true; }
    bool getValue() const { return value_; }

private:
    bool value_;
};

}  // namespace TCLAP

#endif
