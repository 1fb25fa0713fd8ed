// `.ft` scene front-end: lexer, parser, evaluator and lowering to the flat
// scene IR of include/forgedthoughts_gb300.h.
//
// This is a C++ restatement of the subset of the reference language that the
// renderer's hot path consumes (crates/forgedthoughts/src/{lexer,parser,ast,
// eval}.rs): literals, hex colours, let/var bindings, path assignment, object
// literals, `+ - &` on objects, SDF member operators (`union_round`, ...),
// vector arithmetic and builtins, `fn` literals and top-level functions,
// `material`, `environment` and `sdf` blocks, and relative file imports with
// aliases and export lists (crates/forgedthoughts/src/lib.rs:286-1304).
// Layout/skeleton/anchor authoring features are not part of the render hot
// path.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "forgedthoughts_gb300.h"

namespace ftfe {

// ---------------------------------------------------------------- errors
struct FrontendError : std::runtime_error {
  ft_status status;
  FrontendError(ft_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// ------------------------------------------------------------------- AST
// Mirrors crates/forgedthoughts/src/ast.rs.
struct Expr;
using ExprP = std::shared_ptr<const Expr>;

struct FnStmt {  // MaterialFunctionStatement (ast.rs:44-48)
  bool is_return = false;
  std::string name;
  ExprP expr;
};

struct Expr {
  enum Kind { Number, String, Array, FunctionLiteral, Ident, ObjectLiteral, Binary, Member, Call, Unary };
  Kind kind = Number;
  double number = 0.0;
  std::string text;  // string literal, identifier, object type name, member field
  std::vector<ExprP> items;  // array items, call args
  std::vector<std::pair<std::string, ExprP>> fields;  // object literal fields
  std::vector<std::string> params;  // function literal
  std::vector<FnStmt> body;
  ExprP lhs, rhs;  // binary operands; unary operand in lhs; member target / callee in lhs
  char op = 0;     // '+', '-', '&', '*', '/' (binary), '-' (unary)
};

struct BlockStmt {  // MaterialStatement / SdfStatement (ast.rs:50-80)
  enum Kind { Binding, Property, Function };
  Kind kind = Binding;
  std::string name;
  ExprP expr;
  std::vector<std::string> params;
  std::vector<FnStmt> body;
};

struct BlockDef {  // MaterialDef / SdfDef / EnvironmentDef
  std::string name;
  std::string model;  // materials only, default "Standard"
  std::vector<BlockStmt> statements;
};

struct FunctionDef {
  std::string name;
  std::vector<std::string> params;
  std::vector<FnStmt> body;
};

struct Stmt {  // Statement (ast.rs:108-130)
  enum Kind { Import, Export, Binding, Assign, Function, Material, Sdf, Skeleton, Environment };
  Kind kind = Binding;
  std::string name;   // bound name; the path of an import
  std::string alias;  // `import "..." as alias;` (empty: none)
  bool mutable_ = false;
  ExprP expr;
  std::vector<std::string> path;
  std::shared_ptr<FunctionDef> fn;
  std::shared_ptr<BlockDef> block;
};

std::vector<Stmt> parse_program(const std::string& source);

// An asset library item (`BuiltinLibraryItem`, lib.rs:54-61).
struct LibraryItem {
  std::string name, path, source;
};

// Reads `scene_path` and splices every `import` in place, recursively:
// relative paths resolve from the importing file's directory, other paths
// and names select an item of `library`, an import with `as alias` has its
// top-level names qualified as `alias.name`, a file with `export { ... }`
// contributes only the exported names and what they depend on, and a file
// is spliced once per (file, alias) pair.  Throws FrontendError with
// FT_ERR_IO, FT_ERR_MISSING_IMPORT, FT_ERR_IMPORT_CYCLE,
// FT_ERR_AMBIGUOUS_IMPORT, FT_ERR_UNSUPPORTED (a library import with no
// library given) or FT_ERR_PARSE.
std::vector<Stmt> load_program_with_imports(const std::string& scene_path,
                                            const std::vector<LibraryItem>* library = nullptr);

// `a.b.c` as the dotted name "a.b.c" (false for any other expression).  A
// qualified name from an aliased import is looked up this way.
bool flatten_member(const Expr& e, std::string* out);

// ----------------------------------------------------------------- values
// Mirrors `enum Value` (E:22-28).  Objects and arrays are shared and copied on
// write, so building deep boolean trees stays linear.
struct Value;
struct ObjectData;
struct FunctionData;

struct Value {
  enum Kind { Number, String, Array, Object, Function };
  Kind kind = Number;
  float num = 0.0f;
  std::string str;
  std::shared_ptr<std::vector<Value>> arr;
  std::shared_ptr<ObjectData> obj;
  std::shared_ptr<FunctionData> fn;

  static Value number(float v) { Value r; r.kind = Number; r.num = v; return r; }
  bool is_number() const { return kind == Number; }
  bool is_object() const { return kind == Object; }
};

struct ObjectData {
  bool has_type = false;
  std::string type_name;
  std::map<std::string, Value> fields;
  const Value* get(const std::string& k) const {
    auto it = fields.find(k);
    return it == fields.end() ? nullptr : &it->second;
  }
};

struct FunctionData {
  std::vector<std::string> params;
  std::vector<FnStmt> body;
  std::map<std::string, Value> captures;
  uint64_t identity = 0;  // distinct per function literal evaluation site + captures
};

Value make_object(const std::string& type_name, std::map<std::string, Value> fields);
Value make_vec3(float x, float y, float z);
bool as_vec3(const Value& v, float out[3]);
bool as_broadcast_vec3(const Value& v, float out[3]);
bool values_equal(const Value& a, const Value& b);

struct Binding {
  bool mutable_ = false;
  Value value;
};

struct EvalState {  // E:71-88 (render-relevant part)
  std::map<std::string, Binding> bindings;
  std::map<std::string, std::shared_ptr<FunctionDef>> function_defs;
  std::map<std::string, std::shared_ptr<BlockDef>> material_defs;
  std::map<std::string, std::shared_ptr<BlockDef>> sdf_defs;
  std::map<std::string, std::shared_ptr<BlockDef>> environment_defs;
};

EvalState eval_program(const std::vector<Stmt>& program);

// Evaluation helpers shared with the lowering step.
Value eval_builtin(const std::string& name, const std::vector<Value>& args, bool* found);

// Layout member operators and anchor symbols (frontend_layout.cpp).
bool is_anchor_symbol(const std::string& name);
Value anchor_symbol(const std::string& name, float offset);
// `Top + 0.3`: an anchor symbol with an offset; false for other operands.
bool anchor_arithmetic(const Value& l, char op, const Value& r, Value* out);
bool is_layout_member_operator(const std::string& field);
Value build_layout_member(const std::string& field, Value base, const std::vector<Value>& args);

// ---------------------------------------------------------------- lowering
// Owned storage behind an ft_scene_desc returned to C callers.
struct OwnedSceneDesc {
  ft_scene_desc desc{};
  std::vector<ft_node> nodes;
  std::vector<ft_instr> instrs;
  std::vector<ft_program> programs;
  std::vector<ft_light> lights;
  std::vector<ft_material> materials;
  void finalize();  // point desc at the vectors
};

std::unique_ptr<OwnedSceneDesc> lower_scene(const EvalState& state);

}  // namespace ftfe
