// Shared declarations for the reference oracle wrapper (test infrastructure only).
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>

#include <vamp/vector.hh>
#include <vamp/collision/environment.hh>
#include <vamp/collision/validity.hh>
#include <vamp/planning/validate.hh>

// A scalar environment as users build it (collision::Environment<float>) plus the 8-lane copy the
// reference converts it into before each query (bindings/robot_helper.hh:166,252,266,289).
struct RefEnv
{
    vamp::collision::Environment<float> scalar;
    std::unique_ptr<vamp::collision::Environment<vamp::FloatVector<vamp::FloatVectorWidth>>> vec;
    bool dirty = true;
    int n_added = 0;  // objects are named by their insertion order ("0", "1", ...)

    void finalize()
    {
        if (dirty or not vec)
        {
            scalar.sort();
            vec = std::make_unique<vamp::collision::Environment<vamp::FloatVector<vamp::FloatVectorWidth>>>(
                scalar);
            dirty = false;
        }
    }
};
