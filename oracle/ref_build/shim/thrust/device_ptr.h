#pragma once
/* Host-build stand-in: included but unused by the reference sources. */
