/* A project-written stand-in for the structures of OpenTimer's Parser-SPEF
 * that the reference's Parasitics::toSPEF fills (src/solnoutclass.hpp:
 * 1972-2091).  The library is not in the image.  dump() writes the fields
 * one per line in a plain layout of this stand-in's own (not Parser-SPEF's
 * SPEF rendering), so that tests can read back which elements the
 * reference's code chose and their values.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef G2P_PARSER_SPEF_STANDIN_HPP
#define G2P_PARSER_SPEF_STANDIN_HPP

#include <cstdio>
#include <ostream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace spef {

enum class ConnectionDirection { INPUT, OUTPUT, INOUT };
enum class ConnectionType { INTERNAL, EXTERNAL };

struct Port {
    std::string name;
    ConnectionDirection direction = ConnectionDirection::INOUT;
    Port() {}
    Port(const std::string &n) : name(n) {}
};

struct Connection {
    std::string name;
    ConnectionType type = ConnectionType::INTERNAL;
    ConnectionDirection direction = ConnectionDirection::INOUT;
};

struct Net {
    std::string name;
    double lcap = 0;
    std::vector<Connection> connections;
    std::vector<std::tuple<std::string, std::string, double>> caps;
    std::vector<std::tuple<std::string, std::string, double>> ress;
};

struct Spef {
    std::string standard, design_name, date, vendor, program, version, design_flow, divider, delimiter,
        bus_delimiter, time_unit, capacitance_unit, resistance_unit, inductance_unit;
    std::unordered_map<size_t, std::string> name_map;
    std::vector<Port> ports;
    std::vector<Net> nets;

    void dump(std::ostream &os) const {
        char b[64];
        os << "standard " << standard << "\ndesign " << design_name << "\nunits " << time_unit << "|"
           << capacitance_unit << "|" << resistance_unit << "|" << inductance_unit << "\n";
        for (size_t i = 1; i <= name_map.size(); i++) {
            auto it = name_map.find(i);
            if (it != name_map.end()) os << "name " << i << " " << it->second << "\n";
        }
        for (const auto &p : ports) os << "port " << p.name << " " << (int)p.direction << "\n";
        for (const auto &n : nets) {
            std::snprintf(b, sizeof b, "%.17g", n.lcap);
            os << "net " << n.name << " " << b << "\n";
            for (const auto &c : n.connections) os << "conn " << c.name << " " << (int)c.type << " " << (int)c.direction << "\n";
            for (const auto &c : n.caps) {
                std::snprintf(b, sizeof b, "%.17g", std::get<2>(c));
                os << "cap " << std::get<0>(c) << " " << (std::get<1>(c).empty() ? "-" : std::get<1>(c)) << " " << b << "\n";
            }
            for (const auto &r : n.ress) {
                std::snprintf(b, sizeof b, "%.17g", std::get<2>(r));
                os << "res " << std::get<0>(r) << " " << (std::get<1>(r).empty() ? "-" : std::get<1>(r)) << " " << b << "\n";
            }
        }
    }
};

}  // namespace spef

#endif
