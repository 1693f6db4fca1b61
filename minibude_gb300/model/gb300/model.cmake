# model.cmake -- registration of the GB300 model with the reference's CMake model registry
# (cmake/register_models.cmake: register_flag_*, setup(), setup_target(), register_link_library).
#
# Copy this directory to <miniBUDE>/src/gb300/, add `register_model(gb300 GB300 fasten.hpp)` to the
# reference's CMakeLists.txt next to the other register_model lines and, before the `#else` of
# src/main.cpp's model selection chain, the branch
#     #elif defined(GB300)
#       #include "gb300/fasten.hpp"
# then configure with -DMODEL=gb300 -DGB300_ROOT=<this checkout>.
#
# main.cpp stays pure C++ and is compiled by the C++ compiler.  The CUDA sources are compiled by
# nvcc through custom commands into libbude_gb300.so, which the driver links; CMake's CUDA language
# is not enabled, because the reference's CMakeLists.txt escapes the commas of USE_PPWI for nvcc
# whenever CMAKE_CUDA_COMPILER is nvcc, which only a main.cpp compiled by nvcc would accept.

register_flag_required(GB300_ROOT
        "Path of the minibude-gb300 checkout (the directory holding include/ and minibude_gb300/csrc/)")

register_flag_optional(GB300_NVCC
        "The nvcc that compiles the GB300 kernels (CUDA 13 or newer, for sm_103a)"
        "nvcc")

# The translation units of libbude_gb300.so (minibude_gb300/build.py builds the same list).
set(GB300_CU_SOURCES bude_gb300 autotune batch surrogate screen noalloc stream arch_probe)

macro(setup)
    set(CMAKE_CXX_STANDARD 17)
    find_program(GB300_NVCC_PATH NAMES ${GB300_NVCC} nvcc HINTS /usr/local/cuda/bin REQUIRED)
    set(GB300_CSRC ${GB300_ROOT}/minibude_gb300/csrc)
    file(GLOB GB300_HEADERS ${GB300_CSRC}/*.cuh ${GB300_CSRC}/*.h ${GB300_ROOT}/include/*.h)
    set(GB300_NVCC_FLAGS -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17 -Xcompiler -fPIC
            --expt-relaxed-constexpr)
    set(GB300_OBJECTS)
    foreach (GB300_TU ${GB300_CU_SOURCES})
        set(GB300_OBJ ${CMAKE_BINARY_DIR}/gb300/${GB300_TU}.o)
        add_custom_command(OUTPUT ${GB300_OBJ}
                COMMAND ${CMAKE_COMMAND} -E make_directory ${CMAKE_BINARY_DIR}/gb300
                COMMAND ${GB300_NVCC_PATH} ${GB300_NVCC_FLAGS} -c ${GB300_CSRC}/${GB300_TU}.cu -o ${GB300_OBJ}
                DEPENDS ${GB300_CSRC}/${GB300_TU}.cu ${GB300_HEADERS}
                COMMENT "nvcc ${GB300_TU}.cu (sm_103a)"
                VERBATIM)
        list(APPEND GB300_OBJECTS ${GB300_OBJ})
    endforeach ()
    set(GB300_LIB ${CMAKE_BINARY_DIR}/libbude_gb300.so)
    add_custom_command(OUTPUT ${GB300_LIB}
            COMMAND ${GB300_NVCC_PATH} -gencode arch=compute_103a,code=sm_103a -shared -o ${GB300_LIB} ${GB300_OBJECTS}
            DEPENDS ${GB300_OBJECTS}
            COMMENT "link libbude_gb300.so"
            VERBATIM)
    add_custom_target(bude_gb300_build DEPENDS ${GB300_LIB})
    add_library(bude_gb300 SHARED IMPORTED)
    set_target_properties(bude_gb300 PROPERTIES IMPORTED_LOCATION ${GB300_LIB} IMPORTED_NO_SONAME ON)
    include_directories(${GB300_ROOT}/include)
    register_link_library(bude_gb300)
endmacro()

macro(setup_target NAME)
    add_dependencies(${NAME} bude_gb300_build)
    set_target_properties(${NAME} PROPERTIES BUILD_RPATH ${CMAKE_BINARY_DIR})
endmacro()
