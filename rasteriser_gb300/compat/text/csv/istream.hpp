// A minimal stand-in for the text-csv reader, covering only what canmom/rasteriser's
// fileloader.cpp uses (`csv_istream(std::istream&)`, `operator>>(float&)` and the stream's truth
// value). Fields are separated by commas and records by newlines. Where text-csv is not installed,
// this lets the reference's own fileloader.cpp compile unmodified, for the drop-in link build and
// for the oracle.
#ifndef RAST_ORACLE_TEXT_CSV_SHIM_HPP
#define RAST_ORACLE_TEXT_CSV_SHIM_HPP

#include <cstdlib>
#include <istream>
#include <string>

namespace text {
namespace csv {

class csv_istream {
public:
    explicit csv_istream(std::istream& in) : in_(in) {}

    // True while another field can be read.
    explicit operator bool() const { return ok_ && in_.good() && in_.peek() != std::char_traits<char>::eof(); }

    csv_istream& operator>>(float& v) {
        std::string field;
        if (!next_field(field)) { ok_ = false; return *this; }
        char* end = nullptr;
        v = std::strtof(field.c_str(), &end);
        if (end == field.c_str()) ok_ = false;
        return *this;
    }

private:
    bool next_field(std::string& out) {
        out.clear();
        int ch;
        bool any = false;
        while ((ch = in_.get()) != std::char_traits<char>::eof()) {
            any = true;
            if (ch == ',' || ch == '\n') break;
            if (ch != '\r') out.push_back(static_cast<char>(ch));
        }
        return any;
    }

    std::istream& in_;
    bool ok_ = true;
};

}  // namespace csv
}  // namespace text

#endif
