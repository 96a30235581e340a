// The CSV text convention of the reference's tables, profiles and schedules
// (I/RreaCsvTextUtil.H): cells are whitespace-trimmed, commas inside quotes
// are protected, a doubled quote inside quotes is one literal quote.
#pragma once

#include <cctype>
#include <string>
#include <vector>

namespace rrea_host::csv {

inline std::string trim(std::string const& s)
{
    std::size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    return s.substr(b, e - b);
}

inline std::vector<std::string> split_cells(std::string const& line)
{
    std::vector<std::string> cells;
    std::string cell;
    bool quoted = false;
    for (std::size_t i = 0; i < line.size(); ++i) {
        char const c = line[i];
        if (c == '"') {
            if (quoted && i + 1 < line.size() && line[i + 1] == '"') {
                cell.push_back('"');
                ++i;
            } else {
                quoted = !quoted;
            }
        } else if (c == ',' && !quoted) {
            cells.push_back(trim(cell));
            cell.clear();
        } else {
            cell.push_back(c);
        }
    }
    cells.push_back(trim(cell));
    return cells;
}

}  // namespace rrea_host::csv
