#include "Teuchos_RCP.hpp"
