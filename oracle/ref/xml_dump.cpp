// Reads a G+Smo XML file with the reference's own parsers and prints its tensor B-spline patches
// and the first MultiPatch section as plain text (test infrastructure only; never shipped):
//   "patch <id> <dim>", per direction "knots <p> <n> t_0 .. t_{n-1}", "coefs <m> <d>" + m rows
//     (gsXml<gsTensorBSpline<d>>::get, src/gsNurbs/gsTensorBSpline.hpp:644-670)
//   "multipatch <parDim> <k>" + "ids i_0 .. i_{k-1}" (the patches section, id_range or id_index)
//   "interface p1 s1 p2 s2 map.. orient.." and "boundary p s", patch ids translated to positions,
//     sorted and without duplicates (internal::getInterfaces / getBoundaries, src/gsIO/gsXml.cpp,
//     and the gsXml<gsMultiPatch> reader, src/gsIO/gsXmlUtils.hpp:968-1050)
// The generic gsFileData front end is not used: in a build without G+Smo's own build system it
// drags in the hierarchical-spline readers, which do not compile here.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <gsCore/gsMultiPatch.h>
#include <gsIO/gsXml.h>
#include <gsNurbs/gsTensorBSpline.h>
#include <gsNurbs/gsTensorBSplineBasis.h>

using namespace gismo;
using internal::gsXmlAttribute;
using internal::gsXmlNode;

namespace gismo {
namespace internal {
void getInterfaces(gsXmlNode* node, const int d, std::map<int, int>& ids, std::vector<boundaryInterface>& result);
void getBoundaries(gsXmlNode* node, std::map<int, int>& ids, std::vector<patchSide>& result);
}  // namespace internal
}  // namespace gismo

template <short_t D>
static void printPatch(gsXmlNode* node, int id) {
    gsTensorBSpline<D>* tb = internal::gsXml<gsTensorBSpline<D>>::get(node);
    std::printf("patch %d %d\n", id, int(D));
    for (short_t k = 0; k < D; ++k) {
        const gsKnotVector<>& kv = tb->basis().knots(k);
        std::printf("knots %d %d", int(kv.degree()), int(kv.size()));
        for (auto it = kv.begin(); it != kv.end(); ++it) std::printf(" %.17g", *it);
        std::printf("\n");
    }
    const gsMatrix<>& c = tb->coefs();
    std::printf("coefs %d %d\n", int(c.rows()), int(c.cols()));
    for (index_t i = 0; i < c.rows(); ++i) {
        for (index_t j = 0; j < c.cols(); ++j) std::printf(j ? " %.17g" : "%.17g", c(i, j));
        std::printf("\n");
    }
    delete tb;
}

int main(int argc, char** argv) {
    if (argc < 2) { std::cerr << "usage: gsxml file.xml\n"; return 2; }
    std::ifstream in(argv[1]);
    std::stringstream ss;
    ss << in.rdbuf();
    std::string text = ss.str();
    std::vector<char> buf(text.begin(), text.end());
    buf.push_back('\0');
    internal::gsXmlTree doc;
    doc.parse<0>(buf.data());
    gsXmlNode* root = doc.first_node("xml");
    if (!root) { std::cerr << "no xml root\n"; return 1; }
    for (gsXmlNode* g = root->first_node("Geometry"); g; g = g->next_sibling("Geometry")) {
        const char* type = g->first_attribute("type")->value();
        gsXmlAttribute* ida = g->first_attribute("id");
        const int id = ida ? std::atoi(ida->value()) : -1;
        if (!std::strcmp(type, "TensorBSpline2")) printPatch<2>(g, id);
        else if (!std::strcmp(type, "TensorBSpline3")) printPatch<3>(g, id);
        else std::printf("unsupported %d %s\n", id, type);
    }
    gsXmlNode* mp = root->first_node("MultiPatch");
    if (!mp) return 0;
    const int d = std::atoi(mp->first_attribute("parDim")->value());
    gsXmlNode* pn = mp->first_node("patches");
    std::istringstream str(pn->value());
    std::vector<int> order;
    std::map<int, int> ids;
    if (!std::strcmp(pn->first_attribute("type")->value(), "id_range")) {
        int a, b;
        str >> a >> b;
        for (int i = a; i <= b; ++i) { ids[i] = i - a; order.push_back(i); }
    } else {
        int c = 0;
        for (int i; str >> i;) { ids[i] = c++; order.push_back(i); }
    }
    std::printf("multipatch %d %d\nids", d, int(order.size()));
    for (int i : order) std::printf(" %d", i);
    std::printf("\n");
    std::vector<patchSide> bnd;
    for (gsXmlNode* c = mp->first_node("boundary"); c; c = c->next_sibling("boundary")) {
        std::vector<patchSide> t;
        internal::getBoundaries(c, ids, t);
        bnd.insert(bnd.end(), t.begin(), t.end());
    }
    std::sort(bnd.begin(), bnd.end());
    bnd.erase(std::unique(bnd.begin(), bnd.end()), bnd.end());
    std::vector<boundaryInterface> ifc;
    for (gsXmlNode* c = mp->first_node("interfaces"); c; c = c->next_sibling("interfaces")) {
        std::vector<boundaryInterface> t;
        internal::getInterfaces(c, d, ids, t);
        ifc.insert(ifc.end(), t.begin(), t.end());
    }
    std::sort(ifc.begin(), ifc.end());
    ifc.erase(std::unique(ifc.begin(), ifc.end()), ifc.end());
    for (const boundaryInterface& it : ifc) {
        std::printf("interface %d %d %d %d", int(it.first().patch), int(it.first().side().index()),
                    int(it.second().patch), int(it.second().side().index()));
        for (index_t i = 0; i < it.dirMap().size(); ++i) std::printf(" %d", int(it.dirMap()(i)));
        for (index_t i = 0; i < it.dirOrientation().size(); ++i) std::printf(" %d", int(it.dirOrientation()(i)));
        std::printf("\n");
    }
    for (const patchSide& b : bnd) std::printf("boundary %d %d\n", int(b.patch), int(b.side().index()));
    return 0;
}
