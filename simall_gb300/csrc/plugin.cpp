// SimAll plugin ABI v1 entry points (plugins/IPlugin.hpp:20-42,
// plugins/SimAllPluginSdk.hpp:36-57,270-292) so core::PluginLoader
// (src/core/PluginLoader.cpp:68-163) can dlopen this library like any other
// plugin: GetPluginAbi() returns 1 and CreatePlugin() returns an object whose
// vtable matches simall::plugins::IPlugin / PluginBase / CategorisedPlugin
// (category Gpu = 23).  The interface has to be laid out exactly like the
// reference's for the loader to call it, so the class declarations below
// restate that layout: the same namespace, virtual functions in the same
// order, the same data member.  The solver itself is reached through the
// C entry points in simall_gpu.h.
#include "simall_gpu.h"

#include <string>

namespace simall::plugins {

inline constexpr int kPluginAbiVersion = 1;

class IPlugin {
public:
    virtual ~IPlugin() = default;
    virtual std::string name() const = 0;
    virtual std::string version() const = 0;
    virtual void on_load() = 0;
    virtual void on_unload() = 0;
    virtual int abi() const { return kPluginAbiVersion; }
};

class PluginBase : public IPlugin {
public:
    PluginBase() = default;
    ~PluginBase() override = default;
    PluginBase(const PluginBase &) = delete;
    PluginBase &operator=(const PluginBase &) = delete;
    std::string name() const override { return "unnamed"; }
    std::string version() const override { return "0.0.0"; }
    void on_load() override {}
    void on_unload() override {}
    int abi() const override { return kPluginAbiVersion; }
};

enum class PluginCategory { Gpu = 23 };

class CategorisedPlugin : public PluginBase {
public:
    explicit CategorisedPlugin(PluginCategory cat) : category_(cat) {}
    [[nodiscard]] PluginCategory category() const { return category_; }

private:
    PluginCategory category_;
};

}  // namespace simall::plugins

namespace {

class GpuPressurePlugin final : public simall::plugins::CategorisedPlugin {
public:
    GpuPressurePlugin() : CategorisedPlugin(simall::plugins::PluginCategory::Gpu) {}
    std::string name() const override { return "simall_gb300_pressure"; }
    std::string version() const override { return "0.1.0"; }
    void on_load() override {}
    void on_unload() override {}
};

}  // namespace

extern "C" __attribute__((visibility("default"))) simall::plugins::IPlugin *CreatePlugin()
{
    return new GpuPressurePlugin();
}

extern "C" __attribute__((visibility("default"))) int GetPluginAbi() { return simall::plugins::kPluginAbiVersion; }
