// mx_standin.cpp -- the mxArray behind oracle/mex/mex.h, and a C interface
// (mh_*) through which tests build the prhs arguments of a gateway call.
//
// TEST INFRASTRUCTURE ONLY. A numeric mxArray owns a zero-initialised host
// buffer of n elements of its class; a struct mxArray (one element) holds
// named fields, each an mxArray it owns.
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "mex.h"

struct mxArray_tag {
    int cls = mxUNKNOWN_CLASS;
    size_t n = 0;
    void* data = nullptr;
    std::vector<std::pair<std::string, mxArray*>> fields;
};

static size_t elem_bytes(int cls)
{
    switch (cls) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    default: return 0;
    }
}

extern "C" {

mxArray* mxGetField(const mxArray* s, mwIndex i, const char* name)
{
    if (!s || i != 0 || s->cls != mxSTRUCT_CLASS) return nullptr;
    for (const auto& f : s->fields)
        if (f.first == name) return f.second;
    return nullptr;
}

void* mxGetData(const mxArray* a) { return a ? a->data : nullptr; }

size_t mxGetNumberOfElements(const mxArray* a) { return a ? a->n : 0; }

double mxGetScalar(const mxArray* a)
{
    if (!a || !a->n || !a->data) return 0.0;
    switch (a->cls) {
    case mxDOUBLE_CLASS: return *(const double*)a->data;
    case mxSINGLE_CLASS: return *(const float*)a->data;
    case mxINT32_CLASS: return *(const int*)a->data;
    case mxUINT32_CLASS: return *(const unsigned*)a->data;
    default: return 0.0;
    }
}

mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID c, mxComplexity)
{
    mxArray* a = new mxArray_tag;
    a->cls = c;
    a->n = m * n;
    a->data = std::calloc(a->n ? a->n : 1, elem_bytes(c) ? elem_bytes(c) : 1);
    return a;
}

// ---- construction and release for the tests (ctypes) ----
mxArray* mh_numeric(int cls, size_t n, const void* src)
{
    mxArray* a = mxCreateNumericMatrix(n, 1, (mxClassID)cls, mxREAL);
    if (src && n) std::memcpy(a->data, src, n * elem_bytes(cls));
    return a;
}

mxArray* mh_struct(void)
{
    mxArray* a = new mxArray_tag;
    a->cls = mxSTRUCT_CLASS;
    a->n = 1;
    return a;
}

void mh_set_field(mxArray* s, const char* name, mxArray* v)
{
    s->fields.emplace_back(name, v);
}

void mh_free(mxArray* a)
{
    if (!a) return;
    for (auto& f : a->fields) mh_free(f.second);
    std::free(a->data);
    delete a;
}

}  // extern "C"
