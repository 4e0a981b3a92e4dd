// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "../chromabase.h"

namespace Chroma {
struct GroupXML_t {
  std::string xml, id, path;
};
GroupXML_t readXMLGroup(XMLReader& xml, const std::string& path, const std::string& type_name);
}  // namespace Chroma
