// Scene files with imports: `import "./x.ft" [as alias];` and
// `export { a, b };`.
//
// Follows the reference loader (crates/forgedthoughts/src/lib.rs):
//   load_program_with_imports / load_import_source   lib.rs:286-383
//   resolve_import                                   lib.rs:385-416
//   namespace_statements / namespace_expr / _path    lib.rs:623-914, 1228-1304
//   collect_export_names / filter_exported_statements lib.rs:916-986
//   statement_dependencies / expr_dependencies       lib.rs:988-1226
//   resolve_builtin_library_name                     lib.rs:432-451
// The reference's built-in library is not part of this front-end: a caller
// passes its items (name, path, source) in; without them an import that is
// not a relative path fails with FT_ERR_UNSUPPORTED.
#include <limits.h>
#include <stdlib.h>
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstring>
#include <fstream>
#include <map>
#include <optional>
#include <set>
#include <sstream>

#include "frontend.h"

namespace ftfe {
namespace {

using NameSet = std::set<std::string>;

[[noreturn]] void load_fail(ft_status s, const std::string& m) { throw FrontendError(s, m); }

std::string qualify(const std::string& alias, const std::string& name) { return alias + "." + name; }

ExprP make(Expr e) { return std::make_shared<const Expr>(std::move(e)); }

// ------------------------------------------------------------ namespacing
// A top-level name of the imported file, used outside a local scope, becomes
// `alias.name` (lib.rs:1228-1291).  Object-literal type names are qualified
// whenever they name a top-level definition; function literals are kept
// as they are.
ExprP ns_expr(const ExprP& e, const std::string& alias, const NameSet& names, const NameSet& local) {
  switch (e->kind) {
    case Expr::Number:
    case Expr::String:
    case Expr::FunctionLiteral:
      return e;
    case Expr::Ident:
      if (names.count(e->text) && !local.count(e->text)) {
        Expr r = *e;
        r.text = qualify(alias, e->text);
        return make(std::move(r));
      }
      return e;
    case Expr::ObjectLiteral: {
      Expr r = *e;
      if (names.count(e->text)) r.text = qualify(alias, e->text);
      for (auto& kv : r.fields) kv.second = ns_expr(kv.second, alias, names, local);
      return make(std::move(r));
    }
    case Expr::Array:
    case Expr::Call: {
      Expr r = *e;
      if (r.lhs) r.lhs = ns_expr(r.lhs, alias, names, local);
      for (ExprP& a : r.items) a = ns_expr(a, alias, names, local);
      return make(std::move(r));
    }
    case Expr::Binary:
    case Expr::Member:
    case Expr::Unary: {
      Expr r = *e;
      r.lhs = ns_expr(r.lhs, alias, names, local);
      if (r.rhs) r.rhs = ns_expr(r.rhs, alias, names, local);
      return make(std::move(r));
    }
  }
  return e;
}

// A function body: parameters and earlier `let`s shadow top-level names.
std::vector<FnStmt> ns_body(const std::vector<FnStmt>& body, const std::string& alias, const NameSet& names,
                            NameSet scope) {
  std::vector<FnStmt> out = body;
  for (FnStmt& s : out) {
    s.expr = ns_expr(s.expr, alias, names, scope);
    if (!s.is_return) scope.insert(s.name);
  }
  return out;
}

std::shared_ptr<BlockDef> ns_block(const BlockDef& def, const std::string& alias, const NameSet& names) {
  auto out = std::make_shared<BlockDef>(def);
  out->name = qualify(alias, def.name);
  NameSet scope;
  for (const BlockStmt& s : def.statements)
    if (s.kind == BlockStmt::Binding) scope.insert(s.name);
  for (BlockStmt& s : out->statements) {
    if (s.kind == BlockStmt::Function) {
      NameSet fn_scope = scope;
      fn_scope.insert(s.params.begin(), s.params.end());
      s.body = ns_body(s.body, alias, names, std::move(fn_scope));
    } else {
      s.expr = ns_expr(s.expr, alias, names, scope);
    }
  }
  return out;
}

bool defines_name(const Stmt& s) {
  switch (s.kind) {
    case Stmt::Binding:
    case Stmt::Function:
    case Stmt::Material:
    case Stmt::Sdf:
    case Stmt::Skeleton:
    case Stmt::Environment:
      return true;
    default:
      return false;
  }
}

// namespace_statements (lib.rs:623-653) and namespace_statement (655-914).
std::vector<Stmt> namespace_statements(std::vector<Stmt> stmts, const std::string& alias) {
  NameSet names;
  for (const Stmt& s : stmts)
    if (defines_name(s)) names.insert(s.name);
  const NameSet none;
  for (Stmt& s : stmts) {
    switch (s.kind) {
      case Stmt::Binding:
        s.name = qualify(alias, s.name);
        s.expr = ns_expr(s.expr, alias, names, none);
        break;
      case Stmt::Assign:
        if (!s.path.empty() && names.count(s.path[0])) s.path[0] = qualify(alias, s.path[0]);
        s.expr = ns_expr(s.expr, alias, names, none);
        break;
      case Stmt::Function: {
        auto fn = std::make_shared<FunctionDef>(*s.fn);
        fn->body = ns_body(fn->body, alias, names, NameSet(fn->params.begin(), fn->params.end()));
        fn->name = qualify(alias, fn->name);
        s.fn = fn;
        s.name = fn->name;
        break;
      }
      case Stmt::Material:
      case Stmt::Sdf:
      case Stmt::Environment:
        s.block = ns_block(*s.block, alias, names);
        s.name = s.block->name;
        break;
      case Stmt::Skeleton:  // its body is not kept by the parser
        s.name = qualify(alias, s.name);
        break;
      case Stmt::Import:
      case Stmt::Export:
        break;
    }
  }
  return stmts;
}

// ----------------------------------------------------------- dependencies
// expr_dependencies (lib.rs:1174-1218): free names an expression reads.  A
// member chain counts as its full dotted name, which is how an aliased
// import's `alias.name` is found again.
void expr_deps(const Expr& e, const NameSet& local, NameSet& out) {
  switch (e.kind) {
    case Expr::Number:
    case Expr::String:
    case Expr::FunctionLiteral:
      return;
    case Expr::Ident:
      if (!local.count(e.text)) out.insert(e.text);
      return;
    case Expr::ObjectLiteral:
      out.insert(e.text);
      for (const auto& kv : e.fields) expr_deps(*kv.second, local, out);
      return;
    case Expr::Member: {
      std::string flat;
      if (flatten_member(e, &flat) && !local.count(flat.substr(0, flat.find('.')))) out.insert(flat);
      return;
    }
    case Expr::Array:
    case Expr::Call:
      if (e.lhs) expr_deps(*e.lhs, local, out);
      for (const ExprP& a : e.items) expr_deps(*a, local, out);
      return;
    case Expr::Binary:
    case Expr::Unary:
      expr_deps(*e.lhs, local, out);
      if (e.rhs) expr_deps(*e.rhs, local, out);
      return;
  }
}

void body_deps(const std::vector<FnStmt>& body, NameSet scope, NameSet& out) {
  for (const FnStmt& s : body) {
    expr_deps(*s.expr, scope, out);
    if (!s.is_return) scope.insert(s.name);
  }
}

// statement_dependencies (lib.rs:988-1172).
NameSet statement_deps(const Stmt& s) {
  NameSet out;
  switch (s.kind) {
    case Stmt::Binding:
    case Stmt::Assign:
      expr_deps(*s.expr, NameSet(), out);
      break;
    case Stmt::Function:
      body_deps(s.fn->body, NameSet(s.fn->params.begin(), s.fn->params.end()), out);
      break;
    case Stmt::Material:
    case Stmt::Sdf:
    case Stmt::Environment: {
      NameSet scope;
      for (const BlockStmt& b : s.block->statements)
        if (b.kind == BlockStmt::Binding) scope.insert(b.name);
      for (const BlockStmt& b : s.block->statements) {
        if (b.kind == BlockStmt::Function) {
          NameSet fn_scope = scope;
          fn_scope.insert(b.params.begin(), b.params.end());
          body_deps(b.body, std::move(fn_scope), out);
        } else {
          expr_deps(*b.expr, scope, out);
        }
      }
      break;
    }
    case Stmt::Skeleton:  // bones and chains name joints; the body is not kept
    case Stmt::Import:
    case Stmt::Export:
      break;
  }
  return out;
}

// collect_export_names (lib.rs:916-926): nullopt when the file exports
// nothing, so that everything stays visible.
std::optional<NameSet> export_names(const std::vector<Stmt>& stmts) {
  std::optional<NameSet> names;
  for (const Stmt& s : stmts) {
    if (s.kind != Stmt::Export) continue;
    if (!names) names.emplace();
    names->insert(s.path.begin(), s.path.end());
  }
  return names;
}

// filter_exported_statements (lib.rs:928-986): keep the exported names and,
// transitively, what their last definitions read; an assignment stays with
// the binding it writes.
std::vector<Stmt> filter_exported(std::vector<Stmt> stmts, const NameSet& exported) {
  std::map<std::string, size_t> by_name;  // the last definition wins
  for (size_t i = 0; i < stmts.size(); ++i)
    if (defines_name(stmts[i])) by_name[stmts[i].name] = i;
  NameSet keep;
  std::vector<std::string> work(exported.begin(), exported.end());
  while (!work.empty()) {
    std::string name = std::move(work.back());
    work.pop_back();
    if (!keep.insert(name).second) continue;
    auto it = by_name.find(name);
    if (it == by_name.end()) continue;
    for (const std::string& dep : statement_deps(stmts[it->second]))
      if (by_name.count(dep)) work.push_back(dep);
  }
  std::vector<Stmt> out;
  for (Stmt& s : stmts) {
    bool kept = defines_name(s) ? keep.count(s.name) > 0
                : s.kind == Stmt::Assign ? !s.path.empty() && keep.count(s.path[0]) > 0
                                         : false;
    if (kept) out.push_back(std::move(s));
  }
  return out;
}

// ------------------------------------------------------------------ loader
bool starts_with(const std::string& s, const char* p) { return s.rfind(p, 0) == 0; }

std::string directory_of(const std::string& canonical_path) {
  size_t k = canonical_path.find_last_of('/');
  if (k == std::string::npos) return ".";
  return k == 0 ? "/" : canonical_path.substr(0, k);
}

// realpath(3); false with errno set when the path does not resolve.
bool canonicalize(const std::string& path, std::string* out) {
  char buf[PATH_MAX];
  if (!realpath(path.c_str(), buf)) return false;
  *out = buf;
  return true;
}

std::string read_file(const std::string& path) {
  struct stat sb;
  if (stat(path.c_str(), &sb) == 0 && S_ISDIR(sb.st_mode))
    load_fail(FT_ERR_IO, "failed to read scene file " + path + ": " + std::strerror(EISDIR));
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) load_fail(FT_ERR_IO, "failed to read scene file " + path + ": " + std::strerror(errno));
  std::ostringstream ss;
  ss << f.rdbuf();
  if (f.bad()) load_fail(FT_ERR_IO, "failed to read scene file " + path);
  return ss.str();
}

// An import's identity (`ImportKey`, lib.rs:293-297): a file's canonical
// path, or "builtin:" + a library item's path, which is also how a cycle
// report names it (lib.rs:418-422).
const char kBuiltin[] = "builtin:";

struct Loader {
  const std::vector<LibraryItem>* library = nullptr;
  // (key, alias) pairs already spliced (lib.rs:321); "" is "no alias",
  // which no identifier can spell.
  std::set<std::pair<std::string, std::string>> loaded;
  std::vector<std::string> stack;  // keys being loaded, for cycle reports

  const LibraryItem* item_by_path(const std::string& path) const {
    for (const LibraryItem& it : *library)
      if (it.path == path) return &it;
    return nullptr;
  }

  // resolve_import (lib.rs:385-416): relative paths are files; anything
  // else is a library item's path, then a library item's name.
  std::string resolve(const std::string& path, const std::string& base_dir) {
    if (starts_with(path, "./") || starts_with(path, "../")) {
      std::string joined = base_dir + "/" + path, out;
      if (!canonicalize(joined, &out)) {
        if (errno == ENOENT || errno == ENOTDIR)
          load_fail(FT_ERR_MISSING_IMPORT, "missing import '" + path + "' from " + base_dir);
        load_fail(FT_ERR_IO, "failed to read scene file " + joined + ": " + std::strerror(errno));
      }
      return out;
    }
    if (!library)
      load_fail(FT_ERR_UNSUPPORTED, "import '" + path + "' from " + base_dir +
                                        " names the built-in library, which this front-end does not ship;"
                                        " pass the library's items to load it");
    if (item_by_path(path)) return kBuiltin + path;
    std::vector<const LibraryItem*> named;
    for (const LibraryItem& it : *library)
      if (it.name == path) named.push_back(&it);
    if (named.size() == 1) return kBuiltin + named[0]->path;
    if (named.size() > 1) {
      std::string paths;
      for (const LibraryItem* it : named) paths += (paths.empty() ? "" : ", ") + it->path;
      load_fail(FT_ERR_AMBIGUOUS_IMPORT, "ambiguous built-in import '" + path + "' matches: " + paths);
    }
    load_fail(FT_ERR_MISSING_IMPORT, "missing import '" + path + "' from " + base_dir);
  }

  // load_import_source (lib.rs:317-383).
  std::vector<Stmt> load(const std::string& key, const std::string& alias) {
    if (loaded.count({key, alias})) return {};
    if (std::find(stack.begin(), stack.end(), key) != stack.end()) {
      std::string cycle;
      for (const std::string& k : stack) cycle += k + " -> ";
      load_fail(FT_ERR_IMPORT_CYCLE, "import cycle detected: " + cycle + key);
    }
    stack.push_back(key);
    const bool builtin = starts_with(key, kBuiltin);
    // A library item has no directory: its relative imports resolve from
    // the working directory (lib.rs:342, 387).
    const std::string base_dir = builtin ? "." : directory_of(key);
    std::vector<Stmt> program;
    try {
      program = parse_program(builtin ? item_by_path(key.substr(sizeof kBuiltin - 1))->source : read_file(key));
    } catch (const FrontendError& e) {
      if (e.status != FT_ERR_PARSE) throw;
      load_fail(FT_ERR_PARSE, key + ": " + e.what());
    }
    const std::optional<NameSet> exported = export_names(program);
    std::vector<Stmt> stmts;
    for (Stmt& s : program) {
      if (s.kind == Stmt::Import) {
        std::vector<Stmt> sub = load(resolve(s.name, base_dir), s.alias);
        for (Stmt& t : sub) stmts.push_back(std::move(t));
      } else if (s.kind != Stmt::Export) {
        stmts.push_back(std::move(s));
      }
    }
    if (exported) stmts = filter_exported(std::move(stmts), *exported);
    stack.pop_back();
    if (!alias.empty()) stmts = namespace_statements(std::move(stmts), alias);
    loaded.insert({key, alias});
    return stmts;
  }
};

}  // namespace

std::vector<Stmt> load_program_with_imports(const std::string& scene_path, const std::vector<LibraryItem>* library) {
  std::string file;
  if (!canonicalize(scene_path, &file))
    load_fail(FT_ERR_IO, "failed to read scene file " + scene_path + ": " + std::strerror(errno));
  Loader loader;
  loader.library = library;
  return loader.load(file, "");
}

}  // namespace ftfe
