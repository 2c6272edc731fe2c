// Test-infrastructure shim: the reference's headers include this cereal
// header for their serialize() templates. The oracle drives those templates
// with its own capture archive, so nothing from cereal is needed.
#pragma once
