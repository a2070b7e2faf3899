// Formatting hook of the logging shim: nothing to declare.
#pragma once
