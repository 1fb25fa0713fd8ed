// C ABI of the `.ft` front-end: ft_scene_desc_from_source / _from_file /
// ft_scene_desc_free and the thread-local error string shared by every entry
// point.
#include <pthread.h>

#include <cstring>
#include <new>
#include <stdexcept>
#include <system_error>

#include "common.h"
#include "frontend.h"

namespace ftcommon {
namespace {
thread_local std::string g_last_error;
// Set when the message itself could not be stored (no host memory left).
thread_local bool g_last_error_lost = false;
}
void set_last_error(const std::string& message) {
  try {
    g_last_error = message;
    g_last_error_lost = false;
  } catch (...) {
    g_last_error.clear();
    g_last_error_lost = true;
  }
}
void clear_last_error() {
  g_last_error.clear();
  g_last_error_lost = false;
}
const char* last_error_cstr() { return g_last_error_lost ? "out of host memory" : g_last_error.c_str(); }

ft_status fail_current_exception() noexcept {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    return fail(FT_ERR_OUT_OF_MEMORY, "out of host memory");
  } catch (const std::length_error&) {
    return fail(FT_ERR_OUT_OF_MEMORY, "out of host memory (size limit of a host container)");
  } catch (const std::system_error& e) {
    try {
      return fail(FT_ERR_OUT_OF_MEMORY, std::string("host resources exhausted: ") + e.what());
    } catch (...) {
      return fail(FT_ERR_OUT_OF_MEMORY, "host resources exhausted");
    }
  } catch (const std::exception& e) {
    try {
      return fail(FT_ERR_INTERNAL, std::string("internal error: ") + e.what());
    } catch (...) {
      return fail(FT_ERR_INTERNAL, "internal error");
    }
  } catch (...) {
    return fail(FT_ERR_INTERNAL, "internal error: unknown exception");
  }
}
}  // namespace ftcommon

namespace {

struct FrontendJob {
  const char* source = nullptr;  // a scene source, or
  const char* path = nullptr;    // a scene file whose imports are resolved
  const std::vector<ftfe::LibraryItem>* library = nullptr;
  std::unique_ptr<ftfe::OwnedSceneDesc> result;
  ft_status status = FT_OK;
  std::string error;
};

void* run_frontend(void* arg) {
  auto* job = static_cast<FrontendJob*>(arg);
  try {
    std::vector<ftfe::Stmt> program =
        job->path ? ftfe::load_program_with_imports(job->path, job->library) : ftfe::parse_program(job->source);
    ftfe::EvalState state = ftfe::eval_program(program);
    job->result = ftfe::lower_scene(state);
  } catch (const ftfe::FrontendError& e) {
    job->status = e.status;
    job->error = e.what();
  } catch (const std::bad_alloc&) {
    job->status = FT_ERR_OUT_OF_MEMORY;
    job->error = "out of host memory in the scene front-end";
  } catch (const std::exception& e) {
    job->status = FT_ERR_EVAL;
    job->error = e.what();
  } catch (...) {
    job->status = FT_ERR_INTERNAL;
    job->error = "internal error: unknown exception in the scene front-end";
  }
  return nullptr;
}

ft_status run_frontend_job(FrontendJob& job, ft_scene_desc** out) {
  *out = nullptr;
  // Scenes such as `a + b + c + ...` over thousands of objects nest deeply;
  // the recursive evaluator runs on a thread with a large stack.
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, size_t(512) << 20);
  pthread_t th;
  if (pthread_create(&th, &attr, run_frontend, &job) != 0) {
    pthread_attr_destroy(&attr);
    return ftcommon::fail(FT_ERR_OUT_OF_MEMORY, "could not start the front-end thread");
  }
  pthread_join(th, nullptr);
  pthread_attr_destroy(&attr);
  if (job.status != FT_OK) return ftcommon::fail(job.status, job.error);
  ftfe::OwnedSceneDesc* owned = job.result.release();
  // desc is the first member: the C handle points at it.
  *out = &owned->desc;
  ftcommon::clear_last_error();
  return FT_OK;
}

}  // namespace

extern "C" {

uint32_t ft_abi_version(void) { return FT_ABI_VERSION; }

// The string lives in thread-local storage and stays valid until the next
// call on this thread that sets or clears it.
const char* ft_last_error(void) { return ftcommon::last_error_cstr(); }

ft_status ft_scene_desc_from_source(const char* source, ft_scene_desc** out) {
  FT_API_BEGIN
  if (!source || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "source and out must be non-null");
  FrontendJob job;
  job.source = source;
  return run_frontend_job(job, out);
  FT_API_END
}

ft_status ft_scene_desc_from_file(const char* path, ft_scene_desc** out) {
  return ft_scene_desc_from_file_with_library(path, nullptr, 0, out);
}

ft_status ft_scene_desc_from_file_with_library(const char* path, const ft_library_item* items, uint32_t n_items,
                                               ft_scene_desc** out) {
  FT_API_BEGIN
  if (!path || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "path and out must be non-null");
  if (n_items && !items) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "items is null but n_items is not 0");
  std::vector<ftfe::LibraryItem> library;
  library.reserve(n_items);
  for (uint32_t i = 0; i < n_items; ++i) {
    if (!items[i].name || !items[i].path || !items[i].source)
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT,
                            "library item " + std::to_string(i) + " has a null name, path or source");
    library.push_back({items[i].name, items[i].path, items[i].source});
  }
  FrontendJob job;
  job.path = path;
  job.library = items ? &library : nullptr;
  return run_frontend_job(job, out);
  FT_API_END
}

void ft_scene_desc_free(ft_scene_desc* desc) {
  if (!desc) return;
  auto* owned = reinterpret_cast<ftfe::OwnedSceneDesc*>(reinterpret_cast<char*>(desc) -
                                                         offsetof(ftfe::OwnedSceneDesc, desc));
  delete owned;
}

}  // extern "C"
