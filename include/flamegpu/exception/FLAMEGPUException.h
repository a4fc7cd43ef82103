#ifndef INCLUDE_FLAMEGPU_EXCEPTION_FLAMEGPUEXCEPTION_H_
#define INCLUDE_FLAMEGPU_EXCEPTION_FLAMEGPUEXCEPTION_H_
// Host exception hierarchy with the reference's class names
// (include/flamegpu/exception/FLAMEGPUException.h), so model code and tests
// catch the same types.
#include <cstdarg>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace flamegpu {
namespace exception {

class FLAMEGPUException : public std::exception {
 public:
    explicit FLAMEGPUException(std::string msg = "") : message(std::move(msg)) {}
    const char* what() const noexcept override { return message.c_str(); }
    virtual const char* exception_type() const { return "FLAMEGPUException"; }

 protected:
    std::string message;
};

#define FLAMEGPU_DERIVED_EXCEPTION(name)                                                  \
    class name : public FLAMEGPUException {                                               \
     public:                                                                              \
        explicit name(std::string msg = "") : FLAMEGPUException(std::move(msg)) {}        \
        const char* exception_type() const override { return #name; }                     \
    };

FLAMEGPU_DERIVED_EXCEPTION(CUDAError)
FLAMEGPU_DERIVED_EXCEPTION(InvalidArgument)
FLAMEGPU_DERIVED_EXCEPTION(InvalidAgentVar)
FLAMEGPU_DERIVED_EXCEPTION(InvalidVarType)
FLAMEGPU_DERIVED_EXCEPTION(InvalidAgentName)
FLAMEGPU_DERIVED_EXCEPTION(InvalidAgentState)
FLAMEGPU_DERIVED_EXCEPTION(InvalidAgentFunc)
FLAMEGPU_DERIVED_EXCEPTION(InvalidFuncLayerIndx)
FLAMEGPU_DERIVED_EXCEPTION(InvalidMessage)
FLAMEGPU_DERIVED_EXCEPTION(InvalidMessageName)
FLAMEGPU_DERIVED_EXCEPTION(InvalidMessageVar)
FLAMEGPU_DERIVED_EXCEPTION(InvalidMessageType)
FLAMEGPU_DERIVED_EXCEPTION(InvalidEnvProperty)
FLAMEGPU_DERIVED_EXCEPTION(InvalidEnvPropertyType)
FLAMEGPU_DERIVED_EXCEPTION(InvalidOperation)
FLAMEGPU_DERIVED_EXCEPTION(InvalidHostFunc)
FLAMEGPU_DERIVED_EXCEPTION(InvalidDependencyGraph)
FLAMEGPU_DERIVED_EXCEPTION(OutOfBoundsException)
FLAMEGPU_DERIVED_EXCEPTION(OutOfMemory)
FLAMEGPU_DERIVED_EXCEPTION(UnsupportedVarType)
FLAMEGPU_DERIVED_EXCEPTION(DeviceError)
FLAMEGPU_DERIVED_EXCEPTION(EnsembleError)
FLAMEGPU_DERIVED_EXCEPTION(InvalidConfiguration)
FLAMEGPU_DERIVED_EXCEPTION(ReservedName)
FLAMEGPU_DERIVED_EXCEPTION(JSONError)
FLAMEGPU_DERIVED_EXCEPTION(AgentIDCollision)
FLAMEGPU_DERIVED_EXCEPTION(ArrayMessageWriteConflict)
#undef FLAMEGPU_DERIVED_EXCEPTION

inline std::string format(const char* fmt, ...) {
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return std::string(buf);
}

}  // namespace exception
}  // namespace flamegpu

/** THROW exception::X("fmt", ...) as in the reference. */
#define THROW throw
#endif  // INCLUDE_FLAMEGPU_EXCEPTION_FLAMEGPUEXCEPTION_H_
