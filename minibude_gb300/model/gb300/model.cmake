# model.cmake -- registration of the GB300 model with the reference's CMake model registry
# (cmake/register_models.cmake: register_flag_*, setup(), register_link_library).
#
# Copy this directory to <miniBUDE>/src/gb300/, add `register_model(gb300 GB300 fasten.hpp)` to the
# reference's CMakeLists.txt and the `GB300` branch to src/main.cpp's model selection (the exact
# lines are in INTEGRATION.md), then configure with -DMODEL=gb300 -DGB300_ROOT=<this checkout>.
# main.cpp stays pure C++; the CUDA code is compiled into libbude_gb300 here.

register_flag_required(GB300_ROOT
        "Path of the minibude-gb300 checkout (the directory holding include/ and minibude_gb300/csrc/)")

register_flag_optional(CMAKE_CUDA_COMPILER
        "Path to the CUDA nvcc compiler (CUDA 13 or newer, for sm_103a)"
        "nvcc")

macro(setup)
    set(CMAKE_CXX_STANDARD 17)
    enable_language(CUDA)
    add_library(bude_gb300 SHARED
            ${GB300_ROOT}/minibude_gb300/csrc/bude_gb300.cu
            ${GB300_ROOT}/minibude_gb300/csrc/autotune.cu
            ${GB300_ROOT}/minibude_gb300/csrc/batch.cu
            ${GB300_ROOT}/minibude_gb300/csrc/surrogate.cu
            ${GB300_ROOT}/minibude_gb300/csrc/screen.cu
            ${GB300_ROOT}/minibude_gb300/csrc/noalloc.cu
            ${GB300_ROOT}/minibude_gb300/csrc/stream.cu
            ${GB300_ROOT}/minibude_gb300/csrc/arch_probe.cu)
    target_include_directories(bude_gb300 PUBLIC ${GB300_ROOT}/include)
    target_compile_options(bude_gb300 PRIVATE
            $<$<COMPILE_LANGUAGE:CUDA>:-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17>)
    set_target_properties(bude_gb300 PROPERTIES CUDA_ARCHITECTURES OFF POSITION_INDEPENDENT_CODE ON)
    include_directories(${GB300_ROOT}/include)
    register_link_library(bude_gb300)
endmacro()
