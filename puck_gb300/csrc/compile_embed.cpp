// puck_compile_grammar: the reference's CompileGrammar (src/main/scala/puck/
// parser/CompileGrammar.scala:20-72) behind the C ABI.
//
// The grammar compiler of this library -- the Berkeley text reader, the rule
// buckets, CoarseParent segments, pair tables and backtrace tables, and the
// grammar.grz writer -- is host-side Python over numpy (puck_gb300.berkeley,
// puck_gb300.grammar, puck_gb300.grz, driven by puck_gb300.compile_grammar).
// This entry point runs that same compiler in an embedded CPython
// interpreter, so that a host which binds only this library (a JVM through
// Panama or JNI) compiles grammars exactly as the command-line program does.
// The interpreter's C API is resolved at run time: from the calling process
// when it already hosts Python (a ctypes caller), else from
// libpython3.<minor>.so, which is then initialised once and kept.  The
// library itself does not link against Python.
#include "../../include/puck_gpu.h"
#include "puck_internal.h"

#include <dlfcn.h>

#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

namespace {

// The few CPython entry points used, with their C signatures (PyObject* and
// PyGILState_STATE as opaque handles).
struct PyApi {
  int (*IsInitialized)();
  void (*InitializeEx)(int);
  int (*GILStateEnsure)();
  void (*GILStateRelease)(int);
  void* (*DictNew)();
  void* (*RunString)(const char*, int, void*, void*);
  void* (*DictGetItemString)(void*, const char*);
  long (*LongAsLong)(void*);
  const char* (*UnicodeAsUTF8)(void*);
  void (*DecRef)(void*);
  void (*ErrClear)();
  void* (*EvalSaveThread)();
  bool ok = false;
};

constexpr int kPyFileInput = 257;  // Py_file_input

std::mutex g_py_mu;
PyApi g_py;

template <class F>
bool resolve(void* h, const char* name, F& f) {
  f = reinterpret_cast<F>(dlsym(h, name));
  return f != nullptr;
}

bool load_api(void* h, PyApi& a) {
  return resolve(h, "Py_IsInitialized", a.IsInitialized) && resolve(h, "Py_InitializeEx", a.InitializeEx) &&
         resolve(h, "PyGILState_Ensure", a.GILStateEnsure) && resolve(h, "PyGILState_Release", a.GILStateRelease) &&
         resolve(h, "PyDict_New", a.DictNew) && resolve(h, "PyRun_String", a.RunString) &&
         resolve(h, "PyDict_GetItemString", a.DictGetItemString) && resolve(h, "PyLong_AsLong", a.LongAsLong) &&
         resolve(h, "PyUnicode_AsUTF8", a.UnicodeAsUTF8) && resolve(h, "Py_DecRef", a.DecRef) &&
         resolve(h, "PyErr_Clear", a.ErrClear) && resolve(h, "PyEval_SaveThread", a.EvalSaveThread);
}

// The interpreter: the caller's own, or libpython loaded and initialised here.
bool python(std::string* why) {
  if (g_py.ok) return true;
  PyApi a;
  if (load_api(RTLD_DEFAULT, a) && a.IsInitialized()) {
    g_py = a;
    g_py.ok = true;
    return true;
  }
  const char* names[] = {"libpython3.12.so.1.0", "libpython3.12.so", "libpython3.so"};
  for (const char* n : names) {
    void* h = dlopen(n, RTLD_NOW | RTLD_GLOBAL);
    if (!h) continue;
    if (load_api(h, a)) {
      if (!a.IsInitialized()) {
        a.InitializeEx(0);
        a.EvalSaveThread();  // the initialising thread gives up the GIL; calls take it with PyGILState_Ensure
      }
      g_py = a;
      g_py.ok = true;
      return true;
    }
  }
  *why = "no CPython interpreter: the process hosts none and libpython3.12 could not be loaded";
  return false;
}

// Directory holding the puck_gb300 package: this library is
// <root>/puck_gb300/_build/libpuck_gb300.so.
std::string package_root() {
  Dl_info info{};
  if (!dladdr(reinterpret_cast<void*>(&puck_compile_grammar), &info) || !info.dli_fname) return ".";
  std::string p = info.dli_fname;
  for (int up = 0; up < 3; ++up) {
    const size_t k = p.find_last_of('/');
    if (k == std::string::npos) return ".";
    p.resize(k);
  }
  return p.empty() ? "/" : p;
}

// A Python bytes literal of s (hex), so no quoting can break the script.
std::string py_str(const std::string& s) {
  static const char* hex = "0123456789abcdef";
  std::string out = "bytes.fromhex('";
  for (unsigned char c : s) {
    out += hex[c >> 4];
    out += hex[c & 15];
  }
  return out + "').decode('utf-8')";
}

}  // namespace

extern "C" void puck_default_compile_options(puck_compile_options* o) {
  if (!o) return;
  o->viterbi = 1;
  o->logsum = 0;
  o->reproject = 0;
  o->threshold = -12.0f;
}

extern "C" puck_status puck_compile_grammar(const char* text_prefixes, const char* out_grz,
                                           const puck_compile_options* opts) {
  if (!text_prefixes || !*text_prefixes || !out_grz || !*out_grz) {
    puck::set_last_error("puck_compile_grammar: text_prefixes and out_grz are required");
    return PUCK_ERR_INVALID_ARG;
  }
  puck_compile_options o;
  puck_default_compile_options(&o);
  if (opts) o = *opts;
  std::lock_guard<std::mutex> lk(g_py_mu);
  std::string why;
  if (!python(&why)) {
    puck::set_last_error("puck_compile_grammar: " + why);
    return PUCK_ERR_INTERNAL;
  }
  char thr[64];
  std::snprintf(thr, sizeof thr, "%.9g", (double)o.threshold);
  const std::string code =
      "import sys\n"
      "_root = " + py_str(package_root()) + "\n"
      "if _root not in sys.path:\n"
      "    sys.path.insert(0, _root)\n"
      "try:\n"
      "    from puck_gb300 import compile_grammar as _cg\n"
      "    rc = _cg.main(['--textGrammarPrefix', " + py_str(text_prefixes) + ", '--grammar', " +
      py_str(out_grz) + ", '--viterbi', '" + (o.viterbi ? "true" : "false") + "', '--logsum', '" +
      (o.logsum ? "true" : "false") + "', '--reproject', '" + (o.reproject ? "true" : "false") +
      "', '--threshold', '" + thr + "'])\n"
      "    err = '' if rc == 0 else 'compile_grammar exited with status %d' % rc\n"
      "except SystemExit as e:\n"
      "    rc, err = 2, 'compile_grammar: bad arguments (%s)' % e\n"
      "except Exception as e:\n"
      "    rc, err = 2, '%s: %s' % (type(e).__name__, e)\n";
  const int gil = g_py.GILStateEnsure();
  puck_status st = PUCK_OK;
  std::string msg;
  void* ns = g_py.DictNew();
  void* res = ns ? g_py.RunString(code.c_str(), kPyFileInput, ns, ns) : nullptr;
  if (!res) {
    g_py.ErrClear();
    st = PUCK_ERR_INTERNAL;
    msg = "puck_compile_grammar: the embedded compiler could not run";
  } else {
    g_py.DecRef(res);
    void* rc = g_py.DictGetItemString(ns, "rc");     // borrowed
    void* err = g_py.DictGetItemString(ns, "err");   // borrowed
    const long v = rc ? g_py.LongAsLong(rc) : -1;
    if (v != 0) {
      st = PUCK_ERR_BAD_GRAMMAR;
      const char* e = err ? g_py.UnicodeAsUTF8(err) : nullptr;
      msg = std::string("puck_compile_grammar: ") + (e ? e : "failed");
      g_py.ErrClear();
    }
  }
  if (ns) g_py.DecRef(ns);
  g_py.GILStateRelease(gil);
  if (st != PUCK_OK) puck::set_last_error(msg);
  return st;
}
